// implicit_particles.cuh -- particle kernels of the implicit (theta-scheme)
// path: rotation tensor alpha, moment deposition and the Picard mover.
#pragma once
#include "common.cuh"
#include "types.cuh"
#include "wall_particles.cuh"

namespace pic {

template <typename T, typename FT = double>
__device__ __forceinline__ void gather_node(const GridP& g, int i, int j, int k, T ox, T oy, T oz,
                                            const FT* __restrict__ F, T out[3]) {
    int X[2], Y[2], Z[2];
    T wx[2], wy[2], wz[2];
    node_w(ox, i, g.nx, X, wx); node_w(oy, j, g.ny, Y, wy); node_w(oz, k, g.nz, Z, wz);
    out[0] = out[1] = out[2] = T(0);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                long long id = lin(g, X[a], Y[b], Z[c]);
                T w = wx[a] * wy[b] * wz[c];
                out[0] += T(__ldg(&F[id])) * w;
                out[1] += T(__ldg(&F[g.N + id])) * w;
                out[2] += T(__ldg(&F[2 * g.N + id])) * w;
            }
}

template <typename T, typename FT = double>
__device__ __forceinline__ void gather_cell(const GridP& g, int i, int j, int k, T ox, T oy, T oz,
                                            const FT* __restrict__ F, T out[3]) {
    int X[2], Y[2], Z[2];
    T wx[2], wy[2], wz[2];
    cell_w(ox, i, g.nx, X, wx); cell_w(oy, j, g.ny, Y, wy); cell_w(oz, k, g.nz, Z, wz);
    out[0] = out[1] = out[2] = T(0);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                long long id = lin(g, X[a], Y[b], Z[c]);
                T w = wx[a] * wy[b] * wz[c];
                out[0] += T(__ldg(&F[id])) * w;
                out[1] += T(__ldg(&F[g.N + id])) * w;
                out[2] += T(__ldg(&F[2 * g.N + id])) * w;
            }
}

// evaluateAlphaRotationTensor (PIC++/mover.cpp:851-880).
template <typename T>
__device__ __forceinline__ void alpha_tensor(T beta, const T v[3], T gamma, const T E[3], const T B[3], T al[9]) {
    T G = (beta * (E[0] * v[0] + E[1] * v[1] + E[2] * v[2])) + gamma;
    T bs = beta / G;
    T b2c = bs * bs;
    T den = G * (T(1) + b2c * (B[0] * B[0] + B[1] * B[1] + B[2] * B[2]));
    // FP32: one reciprocal for the nine quotients (within 1 ulp of them);
    // FP64 keeps the divisions of the reference
    const T iden = T(1) / den;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            T r = (i == j ? T(1) : T(0)) + (b2c * B[i] * B[j]);
            if (i != j) {
                int l = 3 - i - j;
                T e = ((i - j + 3) % 3 == 1) ? T(1) : T(-1);   // LeviCivita[j][i][l]
                r -= (bs * e * B[l]);
            }
            if constexpr (sizeof(T) == sizeof(float)) al[3 * i + j] = r * iden;
            else al[3 * i + j] = r / den;
        }
}

// Picard stopping rule of moveParticle (mover.cpp:222-223, 292): the loop
// ends when the momentum change falls below 1e-14 |p| or the displacement
// change below 1e-8 dx, or after three iterations.  For the FP32 push the
// momentum threshold is 4 ulp (1e-14 lies below FP32 resolution, which
// would run every particle through all three iterations although the last
// ones only change rounding).
template <typename T> __device__ __forceinline__ T picard_mom_tol() { return T(1e-14); }
template <> __device__ __forceinline__ float picard_mom_tol<float>() { return 4.8e-7f; }
template <typename T> __device__ __forceinline__ T picard_pos_tol() { return T(1e-8); }

// Picard tests compare a norm with tol x a reference norm; FP32 compares the
// squares (no square roots), FP64 the norms as the reference does.
template <typename T> __device__ __forceinline__ T picard_norm(T sq) {
    if constexpr (sizeof(T) == sizeof(float)) return sq;
    else return dev_sqrt(sq);
}
template <typename T> __device__ __forceinline__ T picard_ref(T x) {   // a reference length in picard_norm's form
    if constexpr (sizeof(T) == sizeof(float)) return x * x;
    else return x;
}
template <typename T> __device__ __forceinline__ T picard_bound(T tol, T ref) {   // ref in picard_norm's form
    if constexpr (sizeof(T) == sizeof(float)) return (tol * tol) * ref;
    else return tol * ref;
}

// The loop test itself: go on while both changes exceed their thresholds
// and fewer than three iterations ran.  The displacement change after the
// first iteration measures the predictor against an iterate that still
// uses the fields at the old position; where FP64 finds it just below
// 1e-8 dx and stops there, FP32 resolves it only to about 3e-8 dx and may
// take the second iteration, whose velocity includes the fields at the mid
// point (measured: up to 2e-5 cells, 3e-7 of the box, for a few hundred of
// 4.2 million gamma = 10 ions of a 64x64x16 box).
template <typename T>
__device__ __forceinline__ bool picard_continue(T err, T momNorm, T cerr, T dxN, int it) {
    return err > picard_bound<T>(picard_mom_tol<T>(), momNorm) && cerr > picard_bound<T>(picard_pos_tol<T>(), dxN) &&
           it < 3;
}

template <typename T>
__device__ __forceinline__ void gamma_vel(const T mom[3], T m, T& gam, T v[3]) {
    T p2 = mom[0] * mom[0] + mom[1] * mom[1] + mom[2] * mom[2];
    gam = dev_sqrt(p2 / (m * m) + T(1));
    if constexpr (sizeof(T) == sizeof(float)) {   // one reciprocal for the three quotients
        const T r = T(1) / (m * gam);
        v[0] = mom[0] * r; v[1] = mom[1] * r; v[2] = mom[2] * r;
    } else {
        v[0] = mom[0] / (m * gam); v[1] = mom[1] / (m * gam); v[2] = mom[2] / (m * gam);
    }
}

// evaluateParticlesRotationTensor (PIC++/mover.cpp:810-841) and the particle
// loops of updateElectroMagneticParameters (PIC++/momentum_collecting.cpp
// 397-584): J-hat, mu to nodes; rho-hat, Pi to cells.  FP64 global atomics.
template <typename T>
__global__ void __launch_bounds__(128) k_implicit_deposit(GridP g, PartView<T> p, double q, double m, double w,
                                                          const double* __restrict__ E, const double* __restrict__ B,
                                                          double* __restrict__ J, double* __restrict__ mu,
                                                          double* __restrict__ rho, double* __restrict__ Pi,
                                                          int compat, GhostAxes ga) {
    const double PI_D = 3.14159265358979323846;
    const double vol = g.dx * g.dy * g.dz;
    const T beta = T(0.5 * q * g.dt / m);
    const double omega = w * g.theta * g.dt * g.dt * 2 * PI_D * q * q / m;
    const double qw = q * w;
    const long long PN = compat ? (long long)ga.cex * ga.cey * ga.cez : g.N;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < p.n;
         n += (long long)gridDim.x * blockDim.x) {
        T mom[3] = {p.px[n], p.py[n], p.pz[n]};
        T gam, v[3];
        gamma_vel<T>(mom, T(m), gam, v);
        int i, j, k;
        decode(g, p.cell[n], i, j, k);
        T ox = p.ox[n], oy = p.oy[n], oz = p.oz[n];
        T e[3], b[3];
        gather_node<T>(g, i, j, k, ox, oy, oz, E, e);
        gather_cell<T>(g, i, j, k, ox, oy, oz, B, b);
        T al[9];
        alpha_tensor<T>(beta, v, gam, e, b, al);
        T vg[3] = {v[0] * gam, v[1] * gam, v[2] * gam};
        double rv[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) rv[a] = double(al[3 * a] * vg[0] + al[3 * a + 1] * vg[1] + al[3 * a + 2] * vg[2]);
        int X[2], Y[2], Z[2];
        T wx[2], wy[2], wz[2];
        node_w(ox, i, g.nx, X, wx); node_w(oy, j, g.ny, Y, wy); node_w(oz, k, g.nz, Z, wz);
        for (int a = 0; a < 2; ++a)
            for (int bb = 0; bb < 2; ++bb)
                for (int c = 0; c < 2; ++c) {
                    if ((!g.y3 && bb) || (!g.z3 && c)) continue;
                    long long id = lin(g, X[a], Y[bb], Z[c]);
                    double corr = double(wx[a]) * double(wy[bb]) * double(wz[c]) / vol;
#pragma unroll
                    for (int d = 0; d < 3; ++d) atomicAdd(&J[d * g.N + id], rv[d] * (qw * corr));
                    double om = omega * corr;
#pragma unroll
                    for (int d = 0; d < 9; ++d) atomicAdd(&mu[d * g.N + id], -(double(al[d]) * om));
                }
        double ten[9];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int c = 0; c < 3; ++c) ten[3 * a + c] = rv[a] * rv[c];
        cell_w(ox, i, g.nx, X, wx); cell_w(oy, j, g.ny, Y, wy); cell_w(oz, k, g.nz, Z, wz);
        // unwrapped x index of the cell stencil for the reference layout
        const int xl = (g.nx > 1) ? ((ox < T(0.5)) ? i - 1 : i) : 0;
        for (int a = 0; a < 2; ++a)
            for (int bb = 0; bb < 2; ++bb)
                for (int c = 0; c < 2; ++c) {
                    if ((!g.y3 && bb) || (!g.z3 && c)) continue;
                    long long id = lin(g, X[a], Y[bb], Z[c]);
                    double corr = double(wx[a]) * double(wy[bb]) * double(wz[c]) / vol;
                    atomicAdd(&rho[id], qw * corr);
                    long long pid;
                    if (compat) {
                        // a wall box mirrors the ghost cell left of the wall
                        // onto the first cell (momentum_collecting.cpp:560-568)
                        const int ux = xl + a;
                        int rx = g.nx > 1 ? ((g.wall && ux < 0) ? -ux - 1 : ux) + ga.gx : 0;
                        int ry = g.ny > 1 ? bb : 0;
                        int rz = g.nz > 1 ? c : 0;
                        pid = ((long long)rz * ga.cey + ry) * ga.cex + rx;
                    } else {
                        pid = id;
                    }
#pragma unroll
                    for (int d = 0; d < 9; ++d) atomicAdd(&Pi[d * PN + pid], qw * corr * ten[d]);
                }
    }
}

// Particle::evaluateVelocity (PIC++/particle.cpp:366-379) with its
// non-relativistic shortcut below p^2 < 1e-4 m^2.
template <typename T>
__device__ __forceinline__ void evaluate_velocity(const T p[3], T m, T v[3]) {
    T p2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    if constexpr (sizeof(T) == sizeof(float)) {   // one reciprocal for the three quotients
        const T r = T(1) / (p2 < T(1e-4) * m * m ? m : dev_sqrt(p2 + m * m));
        v[0] = p[0] * r; v[1] = p[1] * r; v[2] = p[2] * r;
    } else if (p2 < T(1e-4) * m * m) {
        v[0] = p[0] / m; v[1] = p[1] / m; v[2] = p[2] / m;
    } else {
        T gg = dev_sqrt(p2 + m * m) / m;
        v[0] = p[0] / (m * gg); v[1] = p[1] / (m * gg); v[2] = p[2] / (m * gg);
    }
}

// Constants of the implicit mover for one species.
template <typename T>
struct MoverConst {
    T beta, edt, dt, eta, qdt, mm, dxT, redt;
    T id[3];
    int nn[3];
};
template <typename T>
__device__ __forceinline__ MoverConst<T> mover_const(const GridP& g, double q, double m) {
    MoverConst<T> c;
    c.beta = T(0.5 * q * g.dt / m);
    c.edt = T(g.eta * g.dt);
    c.dt = T(g.dt);
    c.eta = T(g.eta);
    c.qdt = T(q * g.dt);
    c.mm = T(m);
    c.dxT = T(g.dx);
    c.redt = T((1.0 - g.eta) * g.dt);
    c.id[0] = T(g.idx); c.id[1] = T(g.idy); c.id[2] = T(g.idz);
    c.nn[0] = g.nx; c.nn[1] = g.ny; c.nn[2] = g.nz;
    return c;
}

// moveParticle (PIC++/mover.cpp:194-491) of particle n: predictor and up to
// three Picard iterations re-gathering E^{n+theta} (nodes) and B^n (cells)
// from the FP64 grids.  alpha is recomputed from E^n, B^n at x^n (what
// evaluateParticlesRotationTensor stored, mover.cpp:810-841).
template <typename T, bool kWall>
__device__ __forceinline__ void implicit_move_particle(const GridP& g, const PartView<T>& p, long long n,
                                                       const MoverConst<T>& c, const double* __restrict__ E,
                                                       const double* __restrict__ B,
                                                       const double* __restrict__ Et) {
    const T beta = c.beta, edt = c.edt, dt = c.dt, eta = c.eta, qdt = c.qdt, mm = c.mm, dxT = c.dxT, redt = c.redt;
    const T id[3] = {c.id[0], c.id[1], c.id[2]};
    const int nn[3] = {c.nn[0], c.nn[1], c.nn[2]};
    int ci[3];
    decode(g, p.cell[n], ci[0], ci[1], ci[2]);
    T u0[3] = {p.ox[n], p.oy[n], p.oz[n]};
    T mom0[3] = {p.px[n], p.py[n], p.pz[n]};
    T gam, v[3];
    gamma_vel<T>(mom0, mm, gam, v);
    T e[3], b[3], al[9];
    gather_node<T>(g, ci[0], ci[1], ci[2], u0[0], u0[1], u0[2], E, e);
    gather_cell<T>(g, ci[0], ci[1], ci[2], u0[0], u0[1], u0[2], B, b);
    alpha_tensor<T>(beta, v, gam, e, b, al);
    gather_node<T>(g, ci[0], ci[1], ci[2], u0[0], u0[1], u0[2], Et, e);
    // b already holds B^n at x^n
    T vxb[3] = {v[1] * b[2] - v[2] * b[1], -v[0] * b[2] + v[2] * b[0], v[0] * b[1] - v[1] * b[0]};
    T pnew[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) pnew[d] = mom0[d] + (e[d] + vxb[d]) * qdt;
    T vnew[3];
    evaluate_velocity<T>(pnew, mm, vnew);
    T mv[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) mv[d] = v[d] * (T(1) - eta) + vnew[d] * eta;
    if constexpr (kWall) {
        if (wall_left_of<T>(ci[0], u0[0], (mv[0] * edt) * id[0])) {
            wall_reflect_trial<T>(g, ci, u0, mv, vnew, mm, edt, redt, id, pnew);
            p.px[n] = pnew[0]; p.py[n] = pnew[1]; p.pz[n] = pnew[2];
            p.ox[n] = u0[0]; p.oy[n] = u0[1]; p.oz[n] = u0[2];
            p.cell[n] = (int)lin(g, ci[0], ci[1], ci[2]);
            return;
        }
    }
    T vh[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
        vh[a] = (al[3 * a] * gam) * v[0] + (al[3 * a + 1] * gam) * v[1] + (al[3 * a + 2] * gam) * v[2];
    const T momNorm = picard_norm<T>(mom0[0] * mom0[0] + mom0[1] * mom0[1] + mom0[2] * mom0[2]);
    T err = picard_norm<T>((mom0[0] - pnew[0]) * (mom0[0] - pnew[0]) + (mom0[1] - pnew[1]) * (mom0[1] - pnew[1]) +
                     (mom0[2] - pnew[2]) * (mom0[2] - pnew[2]));
    const T dxN = picard_ref<T>(dxT);
    T cerr = dxN;
    T newDisp[3] = {mv[0] * edt, mv[1] * edt, mv[2] * edt};
    T prevDisp[3];
    int it = 0;
    bool reflected = false;
    while (picard_continue<T>(err, momNorm, cerr, dxN, it)) {
        ++it;
        T prevMom[3] = {pnew[0], pnew[1], pnew[2]};
#pragma unroll
        for (int d = 0; d < 3; ++d) prevDisp[d] = newDisp[d];
        T re[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) re[a] = al[3 * a] * e[0] + al[3 * a + 1] * e[1] + al[3 * a + 2] * e[2];
#pragma unroll
        for (int d = 0; d < 3; ++d) mv[d] = vh[d] + re[d] * beta;
#pragma unroll
        for (int d = 0; d < 3; ++d) newDisp[d] = mv[d] * edt;
        if constexpr (kWall) {
            if (wall_left_of<T>(ci[0], u0[0], newDisp[0] * id[0])) {
                wall_reflect_trial<T>(g, ci, u0, mv, vnew, mm, edt, redt, id, pnew);
                reflected = true;
                break;
            }
        }
        int tc[3];
        T tu[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            tc[d] = ci[d]; tu[d] = u0[d];
            advance_axis<T>(tu[d], tc[d], newDisp[d] * id[d], nn[d]);
        }
        gather_node<T>(g, tc[0], tc[1], tc[2], tu[0], tu[1], tu[2], Et, e);
        gather_cell<T>(g, tc[0], tc[1], tc[2], tu[0], tu[1], tu[2], B, b);
        T mvxb[3] = {mv[1] * b[2] - mv[2] * b[1], -mv[0] * b[2] + mv[2] * b[0], mv[0] * b[1] - mv[1] * b[0]};
#pragma unroll
        for (int d = 0; d < 3; ++d) pnew[d] = mom0[d] + (e[d] + mvxb[d]) * qdt;
        err = picard_norm<T>((prevMom[0] - pnew[0]) * (prevMom[0] - pnew[0]) + (prevMom[1] - pnew[1]) * (prevMom[1] - pnew[1]) +
                       (prevMom[2] - pnew[2]) * (prevMom[2] - pnew[2]));
        cerr = picard_norm<T>((prevDisp[0] - newDisp[0]) * (prevDisp[0] - newDisp[0]) +
                        (prevDisp[1] - newDisp[1]) * (prevDisp[1] - newDisp[1]) +
                        (prevDisp[2] - newDisp[2]) * (prevDisp[2] - newDisp[2]));
    }
    if (!reflected) {
        if constexpr (kWall) {
            const int o = wall_final_x<T>(g, ci[0], u0[0], (mv[0] * dt) * id[0]);
            if (o == 2) { p.cell[n] = -1; return; }   // escaped through the open boundary
            if (o == 1) pnew[0] = -pnew[0];
#pragma unroll
            for (int d = 1; d < 3; ++d) advance_axis<T>(u0[d], ci[d], (mv[d] * dt) * id[d], nn[d]);
        } else {
#pragma unroll
            for (int d = 0; d < 3; ++d) advance_axis<T>(u0[d], ci[d], (mv[d] * dt) * id[d], nn[d]);
        }
    }
    p.px[n] = pnew[0]; p.py[n] = pnew[1]; p.pz[n] = pnew[2];
    p.ox[n] = u0[0]; p.oy[n] = u0[1]; p.oz[n] = u0[2];
    p.cell[n] = (int)lin(g, ci[0], ci[1], ci[2]);
}

// The mover over every particle of one species (periodic or wall box).
template <typename T, bool kWall>
__global__ void __launch_bounds__(128) k_implicit_push(GridP g, PartView<T> p, double q, double m,
                                                       const double* __restrict__ E, const double* __restrict__ B,
                                                       const double* __restrict__ Et) {
    const MoverConst<T> c = mover_const<T>(g, q, m);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < p.n;
         n += (long long)gridDim.x * blockDim.x) {
        if (p.cell[n] < 0) continue;   // escaped, erased by the next sort
        implicit_move_particle<T, kWall>(g, p, n, c, E, B, Et);
    }
}

// The particles the tiled mover left over (a position it had to gather at
// lay outside its staged block), by the bits of S.defer: one thread per mask
// word, each word read once and cleared for the next step.
template <typename T, bool kWall>
__global__ void __launch_bounds__(128) k_implicit_push_deferred(GridP g, ImpSpecies<T> S,
                                                                const double* __restrict__ E,
                                                                const double* __restrict__ B,
                                                                const double* __restrict__ Et) {
    for (int s = 0; s < S.ns; ++s) {
        const PartView<T> p = S.p[s];
        const MoverConst<T> c = mover_const<T>(g, S.q[s], S.m[s]);
        unsigned* mask = S.defer[s];
        const long long words = (p.n + 31) / 32;
        for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < words;
             w += (long long)gridDim.x * blockDim.x) {
            unsigned bits = mask[w];
            if (!bits) continue;
            mask[w] = 0u;
            while (bits) {
                const long long n = w * 32 + (__ffs(bits) - 1);
                bits &= bits - 1u;
                implicit_move_particle<T, kWall>(g, p, n, c, E, B, Et);
            }
        }
    }
}

}  // namespace pic
