// implicit_grid.cuh -- FP64 grid kernels of the implicit Maxwell solve:
// moment corrections, right part, matrix-free operator, field update.
#pragma once
#include "common.cuh"
#include "implicit_particles.cuh"

namespace pic {

constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------------------
// Pressure tensor fold in the reference's ghosted index space
// (sumCellMatrixParameters{X,Y,Z}, PIC++/momentum_exchange.cpp:1643-1741):
// the reference pairs ghost cell r with r + n + 1; reproduced exactly.
// axis: 0 x, 1 y, 2 z.  One thread per (component, line).
__global__ void k_pi_fold_reference(double* __restrict__ P, GhostAxes ga, int axis) {
    const int ce[3] = {ga.cex, ga.cey, ga.cez};
    const long long PN = (long long)ga.cex * ga.cey * ga.cez;
    const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;   // the two other axes
    const long long lines = (long long)ce[a1] * ce[a2];
    const long long total = lines * 9;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        int d = (int)(t / lines);
        long long l = t - d * lines;
        int u1 = (int)(l % ce[a1]), u2 = (int)(l / ce[a1]);
        auto at = [&](int r) -> double& {
            int c[3];
            c[axis] = r; c[a1] = u1; c[a2] = u2;
            return P[d * PN + ((long long)c[2] * ga.cey + c[1]) * ga.cex + c[0]];
        };
        const int e = ce[axis];
        for (int s = 0; s < 3; ++s) {
            double v = at(e - 1 - s) + at(2 - s);
            at(e - 1 - s) = v;
            at(2 - s) = v;
        }
    }
}

// evaluateDivPressureTensor (PIC++/fields.cpp:3158-3223) at node (i,j,k),
// Pi read through PT(a, b, i, j, k).
template <typename PTf>
__device__ __forceinline__ void div_pi(const GridP& g, int i, int j, int k, PTf PT, double out[3]) {
    for (int col = 0; col < 3; ++col) {
        double rA = (PT(0, col, i, j, k) + PT(0, col, i, j - 1, k) + PT(0, col, i, j, k - 1) + PT(0, col, i, j - 1, k - 1)) * 0.25;
        double lA = (PT(0, col, i - 1, j, k) + PT(0, col, i - 1, j - 1, k) + PT(0, col, i - 1, j, k - 1) + PT(0, col, i - 1, j - 1, k - 1)) * 0.25;
        double bA = 0, fA = 0, tA = 0, boA = 0;
        if (g.y3) {
            bA = (PT(1, col, i, j, k) + PT(1, col, i - 1, j, k) + PT(1, col, i, j, k - 1) + PT(1, col, i - 1, j, k - 1)) * 0.25;
            fA = (PT(1, col, i, j - 1, k) + PT(1, col, i - 1, j - 1, k) + PT(1, col, i, j - 1, k - 1) + PT(1, col, i - 1, j - 1, k - 1)) * 0.25;
        }
        if (g.z3) {
            tA = (PT(2, col, i, j, k) + PT(2, col, i, j - 1, k) + PT(2, col, i - 1, j, k) + PT(2, col, i - 1, j - 1, k)) * 0.25;
            boA = (PT(2, col, i, j, k - 1) + PT(2, col, i, j - 1, k - 1) + PT(2, col, i - 1, j, k - 1) + PT(2, col, i - 1, j - 1, k - 1)) * 0.25;
        }
        // reciprocals from the host: a division is a dozen operations on
        // this GPU's 1/64-rate FP64 pipe
        out[col] = ((rA - lA) * g.idx) + ((bA - fA) * g.idy) + ((tA - boA) * g.idz);
    }
}

// evaluateDivFlux (PIC++/fields.cpp:3060-3156) at cell (i,j,k), J through JF.
template <typename JFf>
__device__ __forceinline__ double div_j(const GridP& g, int i, int j, int k, JFf JF) {
    double rX = (JF(0, i + 1, j, k) + JF(0, i + 1, j + 1, k) + JF(0, i + 1, j, k + 1) + JF(0, i + 1, j + 1, k + 1)) * 0.25;
    double lX = (JF(0, i, j, k) + JF(0, i, j + 1, k) + JF(0, i, j, k + 1) + JF(0, i, j + 1, k + 1)) * 0.25;
    double rY = 0, lY = 0, rZ = 0, lZ = 0;
    if (g.y3) {
        rY = (JF(1, i, j + 1, k) + JF(1, i + 1, j + 1, k) + JF(1, i, j + 1, k + 1) + JF(1, i + 1, j + 1, k + 1)) * 0.25;
        lY = (JF(1, i, j, k) + JF(1, i + 1, j, k) + JF(1, i, j, k + 1) + JF(1, i + 1, j, k + 1)) * 0.25;
    }
    if (g.z3) {
        rZ = (JF(2, i + 1, j, k + 1) + JF(2, i, j, k + 1) + JF(2, i, j + 1, k + 1) + JF(2, i + 1, j + 1, k + 1)) * 0.25;
        lZ = (JF(2, i + 1, j, k) + JF(2, i, j, k) + JF(2, i, j + 1, k) + JF(2, i + 1, j + 1, k)) * 0.25;
    }
    return ((rX - lX) * g.idx) + ((rY - lY) * g.idy) + ((rZ - lZ) * g.idz);
}

__device__ __forceinline__ int gphys(int r, int n) { return n > 1 ? wrap_any(r - 2, n) : 0; }
__device__ __forceinline__ int gcl(int r, int n) { return n > 1 ? r : 0; }

// Reference layout: J-hat on ghosted nodes (n + 5 per axis) = periodic fold
// result minus eta dt div(Pi) (momentum_collecting.cpp:622-631).
__global__ void k_jg_build(GridP g, GhostAxes ga, const double* __restrict__ J, const double* __restrict__ P,
                           double* __restrict__ Jg, int nex, int ney, int nez) {
    const long long JN = (long long)nex * ney * nez;
    const long long PN = (long long)ga.cex * ga.cey * ga.cez;
    const bool single = (g.nx == 1 || !g.y3 || !g.z3);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < JN;
         t += (long long)gridDim.x * blockDim.x) {
        int i = (int)(t % nex);
        long long q = t / nex;
        int j = (int)(q % ney), k = (int)(q / ney);
        long long src = lin(g, gphys(i, g.nx), gphys(j, g.ny), gphys(k, g.nz));
        double out[3] = {0, 0, 0};
        bool edge = (i == 0 || i == nex - 1 || j == 0 || j == ney - 1 || k == 0 || k == nez - 1);
        if (!single && !edge) {
            auto PT = [&](int a, int b, int ii, int jj, int kk) -> double {
                return P[(3 * a + b) * PN + ((long long)gcl(kk, g.nz) * ga.cey + gcl(jj, g.ny)) * ga.cex + gcl(ii, g.nx)];
            };
            div_pi(g, i, j, k, PT, out);
        }
        for (int d = 0; d < 3; ++d) Jg[d * JN + t] = J[d * g.N + src] - out[d] * g.eta * g.dt;
        if (g.wall && i <= ga.gx)   // the wall node and the ghosts left of it (momentum_collecting.cpp:638-646)
            for (int d = 0; d < 3; ++d) Jg[d * JN + t] = 0.0;
    }
}

// Reference layout: rho-hat -= theta dt div(J-hat) (momentum_collecting.cpp
// 645-657), written with one low ghost layer (ext index 0 = reference cell 1).
__global__ void k_rho_ext_reference(GridP g, const double* __restrict__ Jg, int nex, int ney, int nez,
                                    const double* __restrict__ rho, double* __restrict__ rho_ext,
                                    int ex, int ey, int ez) {
    const long long JN = (long long)nex * ney * nez;
    const long long EN = (long long)ex * ey * ez;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < EN;
         t += (long long)gridDim.x * blockDim.x) {
        int i = (int)(t % ex);
        long long q = t / ex;
        int j = (int)(q % ey), k = (int)(q / ey);
        int ri = g.nx > 1 ? i + 1 : 0, rj = g.ny > 1 ? j + 1 : 0, rk = g.nz > 1 ? k + 1 : 0;
        auto JF = [&](int d, int ii, int jj, int kk) -> double {
            return Jg[d * JN + ((long long)gcl(kk, g.nz) * ney + gcl(jj, g.ny)) * nex + gcl(ii, g.nx)];
        };
        double div = div_j(g, ri, rj, rk, JF);
        long long src = lin(g, gphys(ri, g.nx), gphys(rj, g.ny), gphys(rk, g.nz));
        rho_ext[t] = rho[src] - g.dt * g.theta * div;
    }
}

// Interior nodes of the reference-layout J-hat back to the periodic array.
__global__ void k_jg_interior(GridP g, const double* __restrict__ Jg, int nex, int ney, int nez,
                              int gx, int gy, int gz, double* __restrict__ J) {
    const long long JN = (long long)nex * ney * nez;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.N;
         c += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, (int)c, i, j, k);
        long long s = ((long long)(k + gz) * ney + (j + gy)) * nex + (i + gx);
        for (int d = 0; d < 3; ++d) J[d * g.N + c] = Jg[d * JN + s];
    }
}

// Periodic layout: J-hat -= eta dt div(Pi) on the box.
__global__ void k_j_minus_divpi(GridP g, const double* __restrict__ Pi, const double* __restrict__ Jin,
                                double* __restrict__ Jout) {
    const bool single = (g.nx == 1 || !g.y3 || !g.z3);
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.N;
         c += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, (int)c, i, j, k);
        double out[3] = {0, 0, 0};
        if (!single) {
            auto PT = [&](int a, int b, int ii, int jj, int kk) -> double {
                return Pi[(3 * a + b) * g.N + linw(g, ii, jj, kk)];
            };
            div_pi(g, i, j, k, PT, out);
        }
        for (int d = 0; d < 3; ++d) Jout[d * g.N + c] = Jin[d * g.N + c] - out[d] * g.eta * g.dt;
    }
}

// Periodic layout: rho_ext from rho-hat -= theta dt div(J-hat).
__global__ void k_rho_ext_periodic(GridP g, const double* __restrict__ J, const double* __restrict__ rho,
                                   double* __restrict__ rho_ext, int ex, int ey, int ez) {
    // 32-bit index arithmetic (the extended box has fewer than 2^31 cells;
    // 64-bit divisions are long integer sequences)
    const unsigned EN = (unsigned)ex * ey * ez;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < EN; t += gridDim.x * blockDim.x) {
        const unsigned q = t / (unsigned)ex;
        const int i = (int)(t - q * (unsigned)ex);
        const int k = (int)(q / (unsigned)ey), j = (int)(q - (unsigned)k * (unsigned)ey);
        int ii = g.nx > 1 ? i - 1 : 0, jj = g.ny > 1 ? j - 1 : 0, kk = g.nz > 1 ? k - 1 : 0;
        auto JF = [&](int d, int a, int b, int c) -> double { return J[d * g.N + linw(g, a, b, c)]; };
        double div = div_j(g, ii, jj, kk, JF);
        rho_ext[t] = rho[linw(g, ii, jj, kk)] - g.dt * g.theta * div;
    }
}

// createInternalEquation right part (PIC++/fields.cpp:2635-2658), evaluateRotB
// (fields.cpp:2799-2860), evaluateGradDensity (fields.cpp:3229-3259).
__global__ void __launch_bounds__(256) k_maxwell_rhs(GridP g, const double* __restrict__ E, const double* __restrict__ B,
                                                     const double* __restrict__ J, const double* __restrict__ rho_ext,
                                                     int ex, int ey, double* __restrict__ rhs) {
    const double cf = g.cfix, cf2 = g.cfix * g.cfix, td = g.theta * g.dt;
    const double gfac = cf2 * g.theta * g.theta * g.dt * g.dt * 4 * kPi;   // the grad rho term's factor, once
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.N;
         c += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, (int)c, i, j, k);
        const int pi_ = i - 1, pj = j - 1, pk = k - 1;
        auto BF = [&](int d, int a, int b, int cc) -> double { return B[d * g.N + linw(g, a, b, cc)]; };
        auto RH = [&](int a, int b, int cc) -> double {
            return rho_ext[((long long)(g.nz > 1 ? cc + 1 : 0) * ey + (g.ny > 1 ? b + 1 : 0)) * ex + (g.nx > 1 ? a + 1 : 0)];
        };
        double BrX[3], BlX[3], BrY[3], BlY[3], BrZ[3], BlZ[3];
        for (int d = 0; d < 3; ++d) {
            BrX[d] = (BF(d, i, j, k) + BF(d, i, pj, k) + BF(d, i, j, pk) + BF(d, i, pj, pk)) / 4.0;
            BlX[d] = (BF(d, pi_, j, k) + BF(d, pi_, pj, k) + BF(d, pi_, j, pk) + BF(d, pi_, pj, pk)) / 4.0;
            BrY[d] = (BF(d, i, j, k) + BF(d, pi_, j, k) + BF(d, i, j, pk) + BF(d, pi_, j, pk)) / 4.0;
            BlY[d] = (BF(d, i, pj, k) + BF(d, pi_, pj, k) + BF(d, i, pj, pk) + BF(d, pi_, pj, pk)) / 4.0;
            BrZ[d] = (BF(d, i, j, k) + BF(d, pi_, j, k) + BF(d, i, pj, k) + BF(d, pi_, pj, k)) / 4.0;
            BlZ[d] = (BF(d, i, j, pk) + BF(d, pi_, j, pk) + BF(d, i, pj, pk) + BF(d, pi_, pj, pk)) / 4.0;
            if (!g.y3) { BrY[d] = 0; BlY[d] = 0; }
            if (!g.z3) { BrZ[d] = 0; BlZ[d] = 0; }
        }
        double rot[3];
        rot[0] = (BrY[2] - BlY[2]) * g.idy - (BrZ[1] - BlZ[1]) * g.idz;
        rot[1] = (BrZ[0] - BlZ[0]) * g.idz - (BrX[2] - BlX[2]) * g.idx;
        rot[2] = (BrX[1] - BlX[1]) * g.idx - (BrY[0] - BlY[0]) * g.idy;
        double dRX = (RH(i, j, k) + RH(i, pj, k) + RH(i, j, pk) + RH(i, pj, pk)) * 0.25;
        double dLX = (RH(pi_, j, k) + RH(pi_, pj, k) + RH(pi_, j, pk) + RH(pi_, pj, pk)) * 0.25;
        double dRY = (RH(i, j, k) + RH(pi_, j, k) + RH(i, j, pk) + RH(pi_, j, pk)) * 0.25;
        double dLY = (RH(i, pj, k) + RH(pi_, pj, k) + RH(i, pj, pk) + RH(pi_, pj, pk)) * 0.25;
        double dRZ = (RH(i, j, k) + RH(i, pj, k) + RH(pi_, j, k) + RH(pi_, pj, k)) * 0.25;
        double dLZ = (RH(i, j, pk) + RH(i, pj, pk) + RH(pi_, j, pk) + RH(pi_, pj, pk)) * 0.25;
        double grad[3] = {(dRX - dLX) * g.idx, (dRY - dLY) * g.idy, (dRZ - dLZ) * g.idz};
        for (int d = 0; d < 3; ++d)
            rhs[d * g.N + c] = E[d * g.N + c] + (rot[d] * cf - (J[d * g.N + c] * 4 * kPi)) * td - (grad[d] * gfac);
    }
}

// Matrix-free implicit Maxwell operator, the rows of createInternalEquationX/
// Y/Z (PIC++/fields.cpp:1396-1509, 1961-2073, 2521-2633), K = (theta dt c')^2
// (fields.cpp:888).  Factored per node as
//   y_a = c0_a x_a - c1_a (mu x)_a + sum_{+-a} K/da^2 ((mu x)_a - x_a)
//         - sum_{d != a, +-d} K/dd^2 x_a
//         + sum_{d != a} K/(4 da dd) [w_d(++) + w_d(--) - w_d(-+) - w_d(+-)]
// with w = mu x evaluated at the neighbour nodes: the same terms as the
// reference's 37-entry rows regrouped (so FP64 results agree to rounding).
template <typename T>
__device__ __forceinline__ void mu_times(const T* __restrict__ mu, long long N, long long id,
                                         const T* __restrict__ x, T w[3]) {
    T x0 = x[id], x1 = x[N + id], x2 = x[2 * N + id];
#pragma unroll
    for (int a = 0; a < 3; ++a)
        w[a] = mu[(3 * a) * N + id] * x0 + mu[(3 * a + 1) * N + id] * x1 + mu[(3 * a + 2) * N + id] * x2;
}

// The operator in two passes, A x = P x + Q (mu x): this GPU's FP64 rate
// (about 1/64 of FP32) makes the apply arithmetic-bound, so mu x is formed
// once per node (9 operations) instead of at every stencil point that reads
// it (centre, 6 neighbours, 12 corners: about 190 operations per node).
// Pass 1: w_a = sum_b mu_ab x_b.  T: FP64, or FP32 for the inner solve of
// the mixed-precision preconditioner.
// skip (FP32 inner solve, else nullptr): return at once when it is set.
template <typename T>
__global__ void __launch_bounds__(256) k_mu_times(long long N, const T* __restrict__ mu,
                                                  const T* __restrict__ x, T* __restrict__ w,
                                                  const unsigned* __restrict__ skip) {
    if (skip && *skip) return;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N;
         c += (long long)gridDim.x * blockDim.x) {
        T wc[3];
        mu_times<T>(mu, N, c, x, wc);
        w[c] = wc[0]; w[N + c] = wc[1]; w[2 * N + c] = wc[2];
    }
}

// Pass 2: per row a (createInternalEquationX/Y/Z, fields.cpp:1396-1509,
// 1961-2073, 2521-2633): diag x_a - c1 w_a; along axis a K/da^2 (w_a - x_a)
// at both neighbours, along the other axes -K/d^2 x_a; in the (a, d) planes
// K/(4 da dd) (w_d(++) - w_d(+-) - w_d(-+) + w_d(--)).  Periodic box.
template <typename T>
__global__ void __launch_bounds__(256) k_maxwell_stencil(GridP g, OpCoef oc, const T* __restrict__ x,
                                                         const T* __restrict__ w, T* __restrict__ y,
                                                         const unsigned* __restrict__ skip) {
    if (skip && *skip) return;
    const long long N = g.N;
    const int n[3] = {g.nx, g.ny, g.nz};
    const long long st[3] = {1, (long long)g.nx, (long long)g.nx * g.ny};
    double diag64 = 1.0;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
        if (oc.has[ax]) diag64 += 2.0 * oc.kd2[ax];
    const T diag = T(diag64);
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N;
         c += (long long)gridDim.x * blockDim.x) {
        int p[3];
        decode(g, (int)c, p[0], p[1], p[2]);
        long long up[3], dn[3];   // linear offsets of the periodic +1 / -1 neighbours
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            up[ax] = p[ax] + 1 == n[ax] ? -(long long)(n[ax] - 1) * st[ax] : st[ax];
            dn[ax] = p[ax] == 0 ? (long long)(n[ax] - 1) * st[ax] : -st[ax];
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const T* xa = x + a * N + c;
            const T* wa = w + a * N + c;
            const T c1 = T(oc.has[a] ? 1.0 + 2.0 * oc.kd2[a] : 1.0);
            T acc = fma(-c1, wa[0], diag * xa[0]);
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                if (!oc.has[ax]) continue;
                const T xs = xa[up[ax]] + xa[dn[ax]];
                if (ax == a) acc = fma(T(oc.kd2[ax]), (wa[up[ax]] + wa[dn[ax]]) - xs, acc);
                else acc = fma(T(-oc.kd2[ax]), xs, acc);
            }
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (d == a || !oc.has[a] || !oc.has[d]) continue;
                const T* wd = w + d * N + c;
                const T sum = (wd[up[a] + up[d]] - wd[up[a] + dn[d]]) - (wd[dn[a] + up[d]] - wd[dn[a] + dn[d]]);
                acc = fma(T(oc.kx4[a][d]), sum, acc);
            }
            y[a * N + c] = acc;
        }
    }
}

// Pass 2 in FP32 for 3-D boxes whose x and y extents are multiples of ZM_TX
// and ZM_TY (the inner solve of the mixed-precision preconditioner): a block
// owns a ZM_TX x ZM_TY column of cells and ZM_ZC consecutive z planes, and
// marches up z with the planes z - 1, z, z + 1 of x and w (one cell of halo
// in x and y, periodic) rotating through shared memory, so each value is
// read from memory once per block instead of once per stencil point.  Same
// terms as k_maxwell_stencil.
constexpr int ZM_TX = 32, ZM_TY = 8, ZM_ZC = 8;
__global__ void __launch_bounds__(ZM_TX * ZM_TY) k_maxwell_stencil_zm(GridP g, OpCoef oc, const float* __restrict__ x,
                                                                      const float* __restrict__ w,
                                                                      float* __restrict__ y,
                                                                      const unsigned* __restrict__ skip) {
    if (*skip) return;
    constexpr int SX = ZM_TX + 2, SY = ZM_TY + 2, PL = SX * SY;
    __shared__ float sx[3][3][PL], sw[3][3][PL];   // [plane slot][component][y][x]
    const long long N = g.N;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int tx = threadIdx.x % ZM_TX, ty = threadIdx.x / ZM_TX;
    const int i0 = blockIdx.x * ZM_TX, j0 = blockIdx.y * ZM_TY, z0 = blockIdx.z * ZM_ZC;
    const int z1 = z0 + ZM_ZC < nz ? z0 + ZM_ZC : nz;
    const float diag = float(1.0 + 2.0 * (oc.kd2[0] + oc.kd2[1] + oc.kd2[2]));
    float c1[3], kd2[3], kx4[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        c1[a] = float(1.0 + 2.0 * oc.kd2[a]);
        kd2[a] = float(oc.kd2[a]);
#pragma unroll
        for (int d = 0; d < 3; ++d) kx4[a][d] = float(oc.kx4[a][d]);
    }
    // plane z (periodic) of x and w with its halo into slot sl
    auto load = [&](int z, int sl) {
        const int zz = z < 0 ? z + nz : (z >= nz ? z - nz : z);
        for (int e = threadIdx.x; e < PL; e += ZM_TX * ZM_TY) {
            const int hx = e % SX, hy = e / SX;
            int ii = i0 + hx - 1, jj = j0 + hy - 1;
            ii = ii < 0 ? ii + nx : (ii >= nx ? ii - nx : ii);
            jj = jj < 0 ? jj + ny : (jj >= ny ? jj - ny : jj);
            const long long id = ((long long)zz * ny + jj) * nx + ii;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                sx[sl][a][e] = x[a * N + id];
                sw[sl][a][e] = w[a * N + id];
            }
        }
    };
    load(z0 - 1, 0);
    load(z0, 1);
    int sm = 0, sc = 1;   // slots of planes z - 1 and z
    for (int z = z0; z < z1; ++z) {
        const int sp = 3 - sm - sc;   // slot of plane z + 1
        load(z + 1, sp);
        __syncthreads();
        const int slot[3] = {sm, sc, sp};
        // value of field F, component a, at offset (dx, dy, dz) from this cell
        auto X = [&](int a, int dx, int dy, int dz) { return sx[slot[dz + 1]][a][(ty + 1 + dy) * SX + tx + 1 + dx]; };
        auto Wv = [&](int a, int dx, int dy, int dz) { return sw[slot[dz + 1]][a][(ty + 1 + dy) * SX + tx + 1 + dx]; };
        const long long c = ((long long)z * ny + (j0 + ty)) * nx + (i0 + tx);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float acc = fmaf(-c1[a], Wv(a, 0, 0, 0), diag * X(a, 0, 0, 0));
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                const int ux = ax == 0, uy = ax == 1, uz = ax == 2;
                const float xs = X(a, ux, uy, uz) + X(a, -ux, -uy, -uz);
                if (ax == a) acc = fmaf(kd2[ax], (Wv(a, ux, uy, uz) + Wv(a, -ux, -uy, -uz)) - xs, acc);
                else acc = fmaf(-kd2[ax], xs, acc);
            }
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (d == a) continue;
                const int ax_ = a == 0, ay_ = a == 1, az_ = a == 2;
                const int dx_ = d == 0, dy_ = d == 1, dz_ = d == 2;
                const float sum = (Wv(d, ax_ + dx_, ay_ + dy_, az_ + dz_) - Wv(d, ax_ - dx_, ay_ - dy_, az_ - dz_)) -
                                  (Wv(d, -ax_ + dx_, -ay_ + dy_, -az_ + dz_) - Wv(d, -ax_ - dx_, -ay_ - dy_, -az_ - dz_));
                acc = fmaf(kx4[a][d], sum, acc);
            }
            y[a * N + c] = acc;
        }
        __syncthreads();   // every thread is done with slot sm before it is refilled
        sm = sc;
        sc = sp;
    }
}

// Transpose of the operator (k_mu_times + k_maxwell_stencil).  The operator splits as A x = P x + Q (mu x)
// with P and Q constant-coefficient periodic stencils that are symmetric
// (P: the diagonal and the -K/d^2 neighbour couplings; Q: -c1 on the node,
// +K/da^2 along axis a in row a, the K/(4 da dd) corner couplings, whose
// (a, d) and (d, a) blocks coincide), so A^T y = P y + mu^T (Q y) per node.
__global__ void __launch_bounds__(256) k_maxwell_apply_t(GridP g, OpCoef oc, const double* __restrict__ mu,
                                                         const double* __restrict__ y, double* __restrict__ out) {
    const long long N = g.N;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N;
         c += (long long)gridDim.x * blockDim.x) {
        int p[3];
        decode(g, (int)c, p[0], p[1], p[2]);
        const int n[3] = {g.nx, g.ny, g.nz};
        double Py[3], Qy[3];
        double diag = 1.0;
        for (int ax = 0; ax < 3; ++ax)
            if (oc.has[ax]) diag += 2.0 * oc.kd2[ax];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double ya = y[a * N + c];
            const double c1 = oc.has[a] ? 1.0 + 2.0 * oc.kd2[a] : 1.0;
            Py[a] = diag * ya;
            Qy[a] = -c1 * ya;
        }
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            if (!oc.has[ax]) continue;
            for (int s = -1; s <= 1; s += 2) {
                int q[3] = {p[0], p[1], p[2]};
                q[ax] = wrap_any(q[ax] + s, n[ax]);
                const long long cn = lin(g, q[0], q[1], q[2]);
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const double ya = y[a * N + cn];
                    Py[a] -= oc.kd2[ax] * ya;
                    if (a == ax) Qy[a] += oc.kd2[ax] * ya;
                }
            }
        }
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (d == a || !oc.has[a] || !oc.has[d]) continue;
                double sum = 0.0;
                for (int sa = -1; sa <= 1; sa += 2)
                    for (int sd = -1; sd <= 1; sd += 2) {
                        int q[3] = {p[0], p[1], p[2]};
                        q[a] = wrap_any(q[a] + sa, n[a]);
                        q[d] = wrap_any(q[d] + sd, n[d]);
                        const double yd = y[d * N + lin(g, q[0], q[1], q[2])];
                        sum += (sa * sd > 0) ? yd : -yd;
                    }
                Qy[a] += oc.kx4[a][d] * sum;
            }
#pragma unroll
        for (int b = 0; b < 3; ++b)
            out[b * N + c] = Py[b] + mu[b * N + c] * Qy[0] + mu[(3 + b) * N + c] * Qy[1] + mu[(6 + b) * N + c] * Qy[2];
    }
}

// evaluateElectricField (fields.cpp:326-339) and evaluateMagneticField
// (fields.cpp:2717-2738) with evaluateRotEgeneral (fields.cpp:2862-2953).
__global__ void __launch_bounds__(256) k_field_update(GridP g, const double* __restrict__ Et, const double* __restrict__ E,
                                                      const double* __restrict__ B, double* __restrict__ En,
                                                      double* __restrict__ Bn, int doE, int doB) {
    const double itheta = 1.0 / g.theta;   // once per thread: divisions are slow on the FP64 pipe
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.N;
         c += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, (int)c, i, j, k);
        if (doE)
            for (int d = 0; d < 3; ++d) En[d * g.N + c] = (Et[d * g.N + c] - E[d * g.N + c] * (1 - g.theta)) * itheta;
        if (!doB) continue;
        auto EF = [&](int d, int a, int b, int cc) -> double { return Et[d * g.N + linw(g, a, b, cc)]; };
        double rX[3], lX[3], rY[3], lY[3], rZ[3], lZ[3];
        for (int d = 0; d < 3; ++d) {
            rX[d] = (EF(d, i + 1, j, k) + EF(d, i + 1, j + 1, k) + EF(d, i + 1, j, k + 1) + EF(d, i + 1, j + 1, k + 1)) / 4.0;
            lX[d] = (EF(d, i, j, k) + EF(d, i, j + 1, k) + EF(d, i, j, k + 1) + EF(d, i, j + 1, k + 1)) / 4.0;
            rY[d] = (EF(d, i, j + 1, k) + EF(d, i + 1, j + 1, k) + EF(d, i, j + 1, k + 1) + EF(d, i + 1, j + 1, k + 1)) / 4.0;
            lY[d] = (EF(d, i, j, k) + EF(d, i + 1, j, k) + EF(d, i, j, k + 1) + EF(d, i + 1, j, k + 1)) / 4.0;
            rZ[d] = (EF(d, i, j, k + 1) + EF(d, i + 1, j, k + 1) + EF(d, i, j + 1, k + 1) + EF(d, i + 1, j + 1, k + 1)) / 4.0;
            lZ[d] = (EF(d, i, j, k) + EF(d, i + 1, j, k) + EF(d, i, j + 1, k) + EF(d, i + 1, j + 1, k)) / 4.0;
            if (!g.y3) { rY[d] = 0; lY[d] = 0; }
            if (!g.z3) { rZ[d] = 0; lZ[d] = 0; }
        }
        double rot[3];
        rot[0] = (rY[2] - lY[2]) * g.idy - (rZ[1] - lZ[1]) * g.idz;
        rot[1] = (rZ[0] - lZ[0]) * g.idz - (rX[2] - lX[2]) * g.idx;
        rot[2] = (rX[1] - lX[1]) * g.idx - (rY[0] - lY[0]) * g.idy;
        for (int d = 0; d < 3; ++d) Bn[d * g.N + c] = B[d * g.N + c] - rot[d] * (g.cfix * g.dt);
    }
}

}  // namespace pic
