// wall.cuh -- conductor wall at x = 0 and open boundary at x = (nx - 2) dx
// for the implicit path (SUPER_CONDUCTOR_LEFT of PIC++, one rank).
//
// The box keeps its periodic storage of nx cells per row; with GridP::wall
// set the physical domain is nodes 0 .. nx - 2 and cells 0 .. nx - 3:
//   node 0       the wall node (the reference's ghosted index 2),
//   node nx - 2  the open boundary node, node nx - 1 the ghost node beyond
//                it (reference xnumber + 2 and + 3: both rows of
//                createFreeRightEquation, fields.cpp:767-781),
//   cell nx - 2  the ghost cell beyond the open boundary (its field is the
//                boundary's, fields.cpp:2738-2741),
//   cell nx - 1  the ghost cell left of the wall (reference index 1: the
//                first cell's field, fields.cpp:2744-2756; deposits into it
//                are mirrored onto the first cell, momentum_collecting.cpp
//                558-568).
// The periodic index wrap of every stencil then reaches exactly the ghost
// values the reference holds, so the deposit, gather and stencil kernels run
// unchanged; the kernels below apply the boundary rules on the planes
// x = 0, nx - 2 and nx - 1, and the movers reflect and drop particles.
#pragma once
#include "common.cuh"

namespace pic {

// After the particle deposits: J-hat and mu vanish on the wall node
// (momentum_collecting.cpp:496-505); rho-hat and (pi_mirror: Pi of the
// periodic placement; the reference-layout Pi mirrors in its deposit)
// deposited in the ghost cell left of the wall move onto the first cell.
// One thread per (j, k).
__global__ void k_wall_moments(GridP g, double* __restrict__ J, double* __restrict__ mu, double* __restrict__ rho,
                               double* __restrict__ Pi, int pi_mirror) {
    const long long N = g.N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)g.ny * g.nz;
         e += (long long)gridDim.x * blockDim.x) {
        const long long row = e * g.nx;   // cell / node (0, j, k)
        const long long ghost = row + g.nx - 1;
#pragma unroll
        for (int d = 0; d < 3; ++d) J[d * N + row] = 0.0;
#pragma unroll
        for (int d = 0; d < 9; ++d) mu[d * N + row] = 0.0;
        rho[row] += rho[ghost];
        rho[ghost] = 0.0;
        if (!pi_mirror) continue;
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            Pi[d * N + row] += Pi[d * N + ghost];
            Pi[d * N + ghost] = 0.0;
        }
    }
}

// J-hat on the wall node once more after J-hat -= eta dt div Pi
// (momentum_collecting.cpp:638-646).
__global__ void k_wall_zero_j(GridP g, double* __restrict__ J) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)g.ny * g.nz;
         e += (long long)gridDim.x * blockDim.x) {
        const long long row = e * g.nx;
#pragma unroll
        for (int d = 0; d < 3; ++d) J[d * g.N + row] = 0.0;
    }
}

// Right parts of the boundary rows: the wall's Gauss row
// -pi (rho-hat of the four cells right of the node around it, fields.cpp
// 759-760) with E_y = E_z = 0 (createSuperConductorLeftEquation,
// fields.cpp:690-765); the open boundary's constant field on nodes nx - 2
// and nx - 1 (createFreeRightEquation).  rho_ext holds rho-hat with one low
// ghost layer per active axis (ext index = cell + 1).
__global__ void k_wall_rhs(GridP g, const double* __restrict__ rho_ext, int ex, int ey, double er0, double er1,
                           double er2, double* __restrict__ rhs) {
    const long long N = g.N;
    const double PI_D = 3.14159265358979323846;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)g.ny * g.nz;
         e += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(e % g.ny), k = (int)(e / g.ny);
        auto RH = [&](int jj, int kk) { return rho_ext[((long long)(kk + 1) * ey + (jj + 1)) * ex + 1]; };
        const long long row = e * g.nx;
        rhs[row] = -PI_D * (RH(j, k) + RH(j - 1, k) + RH(j, k - 1) + RH(j - 1, k - 1));
        rhs[N + row] = 0.0;
        rhs[2 * N + row] = 0.0;
        const double er[3] = {er0, er1, er2};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            rhs[d * N + row + g.nx - 2] = er[d];
            rhs[d * N + row + g.nx - 1] = er[d];
        }
    }
}

// The boundary rows of the operator, over y = A x of the interior rows:
// wall node E_x(0) - E_x(1), E_y(0), E_z(0); identity rows on nodes nx - 2
// and nx - 1.
template <typename T>
__global__ void k_wall_rows(GridP g, const T* __restrict__ x, T* __restrict__ y, const unsigned* __restrict__ skip) {
    if (skip && *skip) return;
    const long long N = g.N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)g.ny * g.nz;
         e += (long long)gridDim.x * blockDim.x) {
        const long long row = e * g.nx;
        y[row] = x[row] * T(1) + x[row + 1] * T(-1);
        y[N + row] = x[N + row];
        y[2 * N + row] = x[2 * N + row];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            y[d * N + row + g.nx - 2] = x[d * N + row + g.nx - 2];
            y[d * N + row + g.nx - 1] = x[d * N + row + g.nx - 1];
        }
    }
}

// After B^{n+1} = B^n - c' dt rot E^theta: the ghost cell beyond the open
// boundary takes the boundary field, the ghost cell left of the wall the
// first cell's new field (evaluateMagneticField, fields.cpp:2738-2756).
__global__ void k_wall_b(GridP g, double* __restrict__ B, double br0, double br1, double br2) {
    const long long N = g.N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)g.ny * g.nz;
         e += (long long)gridDim.x * blockDim.x) {
        const long long row = e * g.nx;
        const double br[3] = {br0, br1, br2};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            B[d * N + row + g.nx - 2] = br[d];
            B[d * N + row + g.nx - 1] = B[d * N + row];
        }
    }
}

}  // namespace pic
