// yee.cuh -- Yee-lattice field updates of the explicit Buneman/Tristan path.
//
// Bandwidth-bound stencils: one thread per cell, consecutive threads on
// consecutive i (coalesced), neighbour reads served by L1/L2.
#pragma once
#include "common.cuh"

namespace pic {

// tristanEvaluateBhalfStep (PIC++/fields.cpp:21-79) with the curls of
// evaluateBunemanRotE{x,y,z} (fields.cpp:3273-3304):
//   B -= (c' dt / 2) curl E,   Bx at (i, j+1/2, k+1/2) etc.
template <typename T>
__global__ void __launch_bounds__(256) k_yee_b_half(GridP g, const T* __restrict__ E, T* __restrict__ B,
                                                    T cdtd2, T dx, T dy, T dz, T idx, T idy, T idz) {
    const long long N = g.N;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N;
         c += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, (int)c, i, j, k);
        const long long ci = lin(g, wrap_p(i + 1, g.nx), j, k);
        const long long cj = lin(g, i, wrap_p(j + 1, g.ny), k);
        const long long ck = lin(g, i, j, wrap_p(k + 1, g.nz));
        const T* Ex = E; const T* Ey = E + N; const T* Ez = E + 2 * N;
        T ex = Ex[c], ey = Ey[c], ez = Ez[c];
        T rx = T(0);
        if (g.y3) rx += divd<T>(Ez[cj] - ez, dy, idy);
        if (g.z3) rx -= divd<T>(Ey[ck] - ey, dz, idz);
        T ry = -divd<T>(Ez[ci] - ez, dx, idx);
        if (g.z3) ry += divd<T>(Ex[ck] - ex, dz, idz);
        T rz = divd<T>(Ey[ci] - ey, dx, idx);
        if (g.y3) rz -= divd<T>(Ex[cj] - ex, dy, idy);
        // conductor wall (GridP::wall): Bx on nodes 0 .. nx - 2, By and Bz on
        // cells 0 .. nx - 3 (fields.cpp:44-70); the ghost columns keep their
        // values (k_wall_yee_ghosts)
        if (g.wall && i == g.nx - 1) continue;
        B[c] = B[c] - rx * cdtd2;
        if (g.wall && i == g.nx - 2) continue;
        B[N + c] = B[N + c] - ry * cdtd2;
        B[2 * N + c] = B[2 * N + c] - rz * cdtd2;
    }
}

// tristanEvaluateE (PIC++/fields.cpp:81-150), curls evaluateBunemanRotB{x,y,z}
// (fields.cpp:3306-3337):  E += (c' curl B - 4 pi J) dt.
// Conductor wall: Ex on cells 0 .. nx - 3, Ey and Ez on nodes 0 .. nx - 2,
// zero on the wall node and (er1, er2) = E0 on the open boundary node
// (fields.cpp:116-121, 136-141).
template <typename T>
__global__ void __launch_bounds__(256) k_yee_e(GridP g, T* __restrict__ E, const T* __restrict__ B,
                                               const double* __restrict__ J, T cf, T dt,
                                               T dx, T dy, T dz, T idx, T idy, T idz, T er1, T er2) {
    const long long N = g.N;
    const T four_pi = T(4.0 * 3.14159265358979323846);
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N;
         c += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, (int)c, i, j, k);
        const long long ci = lin(g, wrap_m(i - 1, g.nx), j, k);
        const long long cj = lin(g, i, wrap_m(j - 1, g.ny), k);
        const long long ck = lin(g, i, j, wrap_m(k - 1, g.nz));
        const T* Bx = B; const T* By = B + N; const T* Bz = B + 2 * N;
        T bx = Bx[c], by = By[c], bz = Bz[c];
        T rx = T(0);
        if (g.y3) rx += divd<T>(bz - Bz[cj], dy, idy);
        if (g.z3) rx -= divd<T>(by - By[ck], dz, idz);
        T ry = -divd<T>(bz - Bz[ci], dx, idx);
        if (g.z3) ry += divd<T>(bx - Bx[ck], dz, idz);
        T rz = divd<T>(by - By[ci], dx, idx);
        if (g.y3) rz -= divd<T>(bx - Bx[cj], dy, idy);
        if (g.wall) {
            if (i == g.nx - 1) continue;
            if (i == 0) { E[N + c] = T(0); E[2 * N + c] = T(0); }
            if (i == g.nx - 2) { E[N + c] = er1; E[2 * N + c] = er2; }
            if (i != g.nx - 2) E[c] = E[c] + (cf * rx - four_pi * T(J[c])) * dt;
            if (i == 0 || i == g.nx - 2) continue;
        } else {
            E[c] = E[c] + (cf * rx - four_pi * T(J[c])) * dt;
        }
        E[N + c] = E[N + c] + (cf * ry - four_pi * T(J[N + c])) * dt;
        E[2 * N + c] = E[2 * N + c] + (cf * rz - four_pi * T(J[2 * N + c])) * dt;
    }
}

// The ghost column left of a conductor wall (storage column nx - 1) as the
// reference's one-rank exchanges set it (exchangeBuneman{E,B}field,
// fields_exchange.cpp:2537-2661 and counterparts, non-periodic branch):
// zero in the cell-centred Ex, By, Bz, the wall node's Ey, Ez, Bx.  The
// column beyond the open boundary keeps its values.  One thread per (j, k).
template <typename T>
__global__ void k_wall_yee_ghosts(GridP g, T* __restrict__ E, T* __restrict__ B) {
    const long long N = g.N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)g.ny * g.nz;
         e += (long long)gridDim.x * blockDim.x) {
        const long long w = e * g.nx, c = w + g.nx - 1;
        E[c] = T(0); E[N + c] = E[N + w]; E[2 * N + c] = E[2 * N + w];
        B[c] = B[w]; B[N + c] = T(0); B[2 * N + c] = T(0);
    }
}

}  // namespace pic
