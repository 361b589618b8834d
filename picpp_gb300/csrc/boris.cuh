// boris.cuh -- explicit Buneman/Tristan particle kernels: staggered gather,
// Boris push and Umeda zigzag current.
//
// Two forms:
//   * k_boris_push / k_zigzag: one thread per particle, global-memory gather
//     and FP64 global atomics.  Used for the separate phase calls
//     (moveParticles, tristanUpdateFlux) and as the parity baseline.
//   * k_push_deposit_tile (boris_tile.cuh): the fused per-tile kernel of the
//     whole-step path.
#pragma once
#include "common.cuh"
#include "wall_particles.cuh"

namespace pic {

// correlationBunemanEBfieldsWithoutMaps (PIC++/correlation.cpp:441-600).
template <typename TP, typename TF>
__device__ __forceinline__ void yee_gather(const GridP& g, int cell, TP ox, TP oy, TP oz,
                                           const TF* __restrict__ E, const TF* __restrict__ B,
                                           TP e[3], TP b[3]) {
    const long long N = g.N;
    int i, j, k;
    decode(g, cell, i, j, k);
    int nX[2], cX[2], nY[2], cY[2], nZ[2], cZ[2];
    TP wnX[2], wcX[2], wnY[2], wcY[2], wnZ[2], wcZ[2];
    node_w(ox, i, g.nx, nX, wnX); cell_w(ox, i, g.nx, cX, wcX);
    node_w(oy, j, g.ny, nY, wnY); cell_w(oy, j, g.ny, cY, wcY);
    node_w(oz, k, g.nz, nZ, wnZ); cell_w(oz, k, g.nz, cZ, wcZ);
    e[0] = e[1] = e[2] = TP(0); b[0] = b[1] = b[2] = TP(0);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int bb = 0; bb < 2; ++bb)
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                e[0] += TP(__ldg(&E[lin(g, cX[a], nY[bb], nZ[cc])])) * wcX[a] * wnY[bb] * wnZ[cc];
                e[1] += TP(__ldg(&E[N + lin(g, nX[a], cY[bb], nZ[cc])])) * wnX[a] * wcY[bb] * wnZ[cc];
                e[2] += TP(__ldg(&E[2 * N + lin(g, nX[a], nY[bb], cZ[cc])])) * wnX[a] * wnY[bb] * wcZ[cc];
                b[0] += TP(__ldg(&B[lin(g, nX[a], cY[bb], cZ[cc])])) * wnX[a] * wcY[bb] * wcZ[cc];
                b[1] += TP(__ldg(&B[N + lin(g, cX[a], nY[bb], cZ[cc])])) * wcX[a] * wnY[bb] * wcZ[cc];
                b[2] += TP(__ldg(&B[2 * N + lin(g, cX[a], cY[bb], nZ[cc])])) * wcX[a] * wcY[bb] * wnZ[cc];
            }
}

// moveParticleTristan (PIC++/mover.cpp:718-742): half electric kick,
// magnetic rotation with the reference's f = 2/sqrt(1 + t^2) (mover.cpp:738),
// half kick, x += v dt.  Returns the new momentum; advances cell/offset.
template <typename TP>
__device__ __forceinline__ void boris(TP q, TP m, TP dt, TP beta, const TP e[3], const TP b[3],
                                      TP mom[3]) {
    TP s = q * dt * TP(0.5);
    TP dp[3] = {e[0] * s, e[1] * s, e[2] * s};
    mom[0] = mom[0] + dp[0]; mom[1] = mom[1] + dp[1]; mom[2] = mom[2] + dp[2];
    TP p2 = mom[0] * mom[0] + mom[1] * mom[1] + mom[2] * mom[2];
    TP gam = dev_sqrt(p2 / (m * m) + TP(1));
    TP bs = beta / gam;
    TP b2 = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
    TP f = TP(2) / dev_sqrt(TP(1) + bs * bs * b2);
    TP pxb[3] = {mom[1] * b[2] - mom[2] * b[1], -mom[0] * b[2] + mom[2] * b[0], mom[0] * b[1] - mom[1] * b[0]};
    TP tm[3] = {mom[0] + pxb[0] * bs, mom[1] + pxb[1] * bs, mom[2] + pxb[2] * bs};
    TP txb[3] = {tm[1] * b[2] - tm[2] * b[1], -tm[0] * b[2] + tm[2] * b[0], tm[0] * b[1] - tm[1] * b[0]};
    TP fb = f * bs;
    mom[0] += txb[0] * fb + dp[0];
    mom[1] += txb[1] * fb + dp[1];
    mom[2] += txb[2] * fb + dp[2];
}

template <typename TP>
__device__ __forceinline__ void velocity(const TP mom[3], TP m, TP v[3]) {
    TP p2 = mom[0] * mom[0] + mom[1] * mom[1] + mom[2] * mom[2];
    TP gam = dev_sqrt(p2 / (m * m) + TP(1));
    v[0] = mom[0] / (m * gam); v[1] = mom[1] / (m * gam); v[2] = mom[2] / (m * gam);
}

// FP32 forms of the same kinematics with the hardware reciprocal square root:
// m gamma = sqrt(m^2 + p^2), so 1/(m gamma) and beta/gamma = beta m/(m gamma)
// need no division.  Used by the FP32 push (the FP64 path keeps the
// reference's operation sequence).
__device__ __forceinline__ void boris_fast(float q, float m, float dt, float beta, const float e[3], const float b[3],
                                           float mom[3]) {
    const float s = q * dt * 0.5f;
    const float dp[3] = {e[0] * s, e[1] * s, e[2] * s};
    mom[0] += dp[0]; mom[1] += dp[1]; mom[2] += dp[2];
    const float p2 = mom[0] * mom[0] + mom[1] * mom[1] + mom[2] * mom[2];
    const float bs = beta * m * rsqrtf(m * m + p2);
    const float b2 = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
    const float f = 2.0f * rsqrtf(1.0f + bs * bs * b2);
    const float pxb[3] = {mom[1] * b[2] - mom[2] * b[1], -mom[0] * b[2] + mom[2] * b[0], mom[0] * b[1] - mom[1] * b[0]};
    const float tm[3] = {mom[0] + pxb[0] * bs, mom[1] + pxb[1] * bs, mom[2] + pxb[2] * bs};
    const float txb[3] = {tm[1] * b[2] - tm[2] * b[1], -tm[0] * b[2] + tm[2] * b[0], tm[0] * b[1] - tm[1] * b[0]};
    const float fb = f * bs;
    mom[0] += txb[0] * fb + dp[0];
    mom[1] += txb[1] * fb + dp[1];
    mom[2] += txb[2] * fb + dp[2];
}
__device__ __forceinline__ void velocity_fast(const float mom[3], float m, float v[3]) {
    const float r = rsqrtf(m * m + mom[0] * mom[0] + mom[1] * mom[1] + mom[2] * mom[2]);
    v[0] = mom[0] * r; v[1] = mom[1] * r; v[2] = mom[2] * r;
}

// Dispatch: fast forms for FP32 state, reference sequence for FP64.
template <typename TP>
__device__ __forceinline__ void boris_t(TP q, TP m, TP dt, TP beta, const TP e[3], const TP b[3], TP mom[3]) {
    boris<TP>(q, m, dt, beta, e, b, mom);
}
template <>
__device__ __forceinline__ void boris_t<float>(float q, float m, float dt, float beta, const float e[3],
                                               const float b[3], float mom[3]) {
    boris_fast(q, m, dt, beta, e, b, mom);
}
template <typename TP>
__device__ __forceinline__ void velocity_t(const TP mom[3], TP m, TP v[3]) { velocity<TP>(mom, m, v); }
template <>
__device__ __forceinline__ void velocity_t<float>(const float mom[3], float m, float v[3]) { velocity_fast(mom, m, v); }

template <typename TP, typename TF>
__global__ void __launch_bounds__(256) k_boris_push(GridP g, PartView<TP> p, TP q, TP m,
                                                    const TF* __restrict__ E, const TF* __restrict__ B) {
    const TP dt = TP(g.dt);
    const TP beta = q * dt / (TP(2) * m);   // Particle::beta (PIC++/particle.cpp:47)
    const TP idx = TP(g.idx), idy = TP(g.idy), idz = TP(g.idz);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < p.n;
         n += (long long)gridDim.x * blockDim.x) {
        int cell = p.cell[n];
        if (cell < 0) continue;   // escaped through the open boundary, erased by the next sort
        TP ox = p.ox[n], oy = p.oy[n], oz = p.oz[n];
        TP e[3], b[3];
        yee_gather<TP, TF>(g, cell, ox, oy, oz, E, B, e, b);
        TP mom[3] = {p.px[n], p.py[n], p.pz[n]};
        boris<TP>(q, m, dt, beta, e, b, mom);
        p.px[n] = mom[0]; p.py[n] = mom[1]; p.pz[n] = mom[2];
        TP v[3];
        velocity<TP>(mom, m, v);
        int i, j, k;
        decode(g, cell, i, j, k);
        if (g.wall) {
            // the escaped particle keeps its position beyond the open
            // boundary: k_zigzag deposits its current, then marks it
            if (tristan_wall_x<TP>(g, i, ox, (v[0] * dt) * idx) & 1) p.px[n] = -mom[0];
        } else {
            advance_axis<TP>(ox, i, (v[0] * dt) * idx, g.nx);
        }
        advance_axis<TP>(oy, j, (v[1] * dt) * idy, g.ny);
        advance_axis<TP>(oz, k, (v[2] * dt) * idz, g.nz);
        p.ox[n] = ox; p.oy[n] = oy; p.oz[n] = oz;
        p.cell[n] = (int)lin(g, i, j, k);
    }
}

// One axis of the zigzag split (PIC++/momentum_collecting.cpp:91-96,
// 200-221): old position P = X - v dt, relay point R, first-segment shift.
template <typename TP>
__device__ __forceinline__ void zig_axis(TP X, TP v, TP dt, TP d, TP invd, int n, TP& P, TP& R, int& sh,
                                         bool mirror = false) {
    TP prev = X - v * dt;
    // in the cell right of the reflecting wall, moving away from it: an old
    // position left of the wall is mirrored (momentum_collecting.cpp:93-99)
    if (mirror && v > TP(0) && prev < TP(0)) prev = -prev;
    TP r = (X + prev) / TP(2);
    if (n == 1) { P = prev; R = r; sh = 0; return; }
    int s = (int)dev_floor(divd<TP>(prev, d, invd));
    if (s != 0) r = TP(s > 0 ? s : 0) * d;
    P = prev; R = r; sh = s;
}

// The 24 current contributions of one particle (addParticleFluxZigzag,
// PIC++/momentum_collecting.cpp:84-230, 3-D and 2-D branches), handed to a
// sink(component, di, dj, dk, value) with offsets relative to the new cell.
template <typename TP, typename Sink>
__device__ __forceinline__ void zigzag_terms(const GridP& g, TP fcd, TP ox, TP oy, TP oz,
                                             const TP v[3], Sink&& sink, bool wall_cell = false) {
    const TP dt = TP(g.dt), dx = TP(g.dx), dy = TP(g.dy), dz = TP(g.dz);
    const TP idx = TP(g.idx), idy = TP(g.idy), idz = TP(g.idz);
    TP X = ox * dx, Y = oy * dy, Z = oz * dz;
    TP PX, PY, PZ, RX, RY, RZ;
    int si, sj, sk;
    zig_axis<TP>(X, v[0], dt, dx, idx, g.nx, PX, RX, si, wall_cell);
    zig_axis<TP>(Y, v[1], dt, dy, idy, g.ny, PY, RY, sj);
    zig_axis<TP>(Z, v[2], dt, dz, idz, g.nz, PZ, RZ, sk);
    TP Fx1 = divd<TP>(fcd * (RX - PX), dt, TP(1.0 / g.dt));
    TP Fy1 = divd<TP>(fcd * (RY - PY), dt, TP(1.0 / g.dt));
    TP Fz1 = divd<TP>(fcd * (RZ - PZ), dt, TP(1.0 / g.dt));
    TP Fx2 = divd<TP>(fcd * (X - RX), dt, TP(1.0 / g.dt));
    TP Fy2 = fcd * v[1] - Fy1;
    TP Fz2 = fcd * v[2] - Fz1;
    TP Wx1 = divd<TP>(PX + RX, TP(2) * dx, TP(0.5) * idx) - TP(si);
    TP Wy1 = divd<TP>(PY + RY, TP(2) * dy, TP(0.5) * idy) - TP(sj);
    TP Wz1 = divd<TP>(PZ + RZ, TP(2) * dz, TP(0.5) * idz) - TP(sk);
    TP Wx2 = divd<TP>(X + RX, TP(2) * dx, TP(0.5) * idx);
    TP Wy2 = divd<TP>(Y + RY, TP(2) * dy, TP(0.5) * idy);
    TP Wz2 = divd<TP>(Z + RZ, TP(2) * dz, TP(0.5) * idz);
    const bool y3 = g.y3, z3 = g.z3;
    if (!y3) { Wy1 = TP(0); Wy2 = TP(0); }
    if (!z3) { Wz1 = TP(0); Wz2 = TP(0); }
    // first segment at (si, sj, sk)
    sink(0, si, sj, sk, Fx1 * (TP(1) - Wy1) * (TP(1) - Wz1));
    if (y3) sink(0, si, sj + 1, sk, Fx1 * Wy1 * (TP(1) - Wz1));
    if (z3) sink(0, si, sj, sk + 1, Fx1 * (TP(1) - Wy1) * Wz1);
    if (y3 && z3) sink(0, si, sj + 1, sk + 1, Fx1 * Wy1 * Wz1);
    sink(1, si, sj, sk, Fy1 * (TP(1) - Wx1) * (TP(1) - Wz1));
    sink(1, si + 1, sj, sk, Fy1 * Wx1 * (TP(1) - Wz1));
    if (z3) sink(1, si, sj, sk + 1, Fy1 * (TP(1) - Wx1) * Wz1);
    if (z3) sink(1, si + 1, sj, sk + 1, Fy1 * Wx1 * Wz1);
    sink(2, si, sj, sk, Fz1 * (TP(1) - Wx1) * (TP(1) - Wy1));
    if (y3) sink(2, si, sj + 1, sk, Fz1 * (TP(1) - Wx1) * Wy1);
    sink(2, si + 1, sj, sk, Fz1 * Wx1 * (TP(1) - Wy1));
    if (y3) sink(2, si + 1, sj + 1, sk, Fz1 * Wx1 * Wy1);
    // second segment at the new cell
    sink(0, 0, 0, 0, Fx2 * (TP(1) - Wy2) * (TP(1) - Wz2));
    if (y3) sink(0, 0, 1, 0, Fx2 * Wy2 * (TP(1) - Wz2));
    if (z3) sink(0, 0, 0, 1, Fx2 * (TP(1) - Wy2) * Wz2);
    if (y3 && z3) sink(0, 0, 1, 1, Fx2 * Wy2 * Wz2);
    sink(1, 0, 0, 0, Fy2 * (TP(1) - Wx2) * (TP(1) - Wz2));
    sink(1, 1, 0, 0, Fy2 * Wx2 * (TP(1) - Wz2));
    if (z3) sink(1, 0, 0, 1, Fy2 * (TP(1) - Wx2) * Wz2);
    if (z3) sink(1, 1, 0, 1, Fy2 * Wx2 * Wz2);
    sink(2, 0, 0, 0, Fz2 * (TP(1) - Wx2) * (TP(1) - Wy2));
    if (y3) sink(2, 0, 1, 0, Fz2 * (TP(1) - Wx2) * Wy2);
    sink(2, 1, 0, 0, Fz2 * Wx2 * (TP(1) - Wy2));
    if (y3) sink(2, 1, 1, 0, Fz2 * Wx2 * Wy2);
}

template <typename TP>
__global__ void __launch_bounds__(256) k_zigzag(GridP g, PartView<TP> p, TP q, TP m, TP w,
                                                double* __restrict__ J) {
    const TP fcd = q * w / (TP(g.dx) * TP(g.dy) * TP(g.dz));
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < p.n;
         n += (long long)gridDim.x * blockDim.x) {
        int cell = p.cell[n];
        if (cell < 0) continue;
        TP mom[3] = {p.px[n], p.py[n], p.pz[n]};
        TP v[3];
        velocity<TP>(mom, m, v);
        int i, j, k;
        decode(g, cell, i, j, k);
        const TP ox = p.ox[n];
        zigzag_terms<TP>(g, fcd, ox, p.oy[n], p.oz[n], v,
                         [&](int comp, int di, int dj, int dk, TP val) {
                             atomicAdd(&J[comp * g.N + linw(g, i + di, j + dj, k + dk)], double(val));
                         },
                         g.wall && i == kTristanWallNode);
        // eraseEscapedPaticles (mover.cpp:167-192) after the deposit: the
        // next sort drops the particle
        if (g.wall && tristan_escaped<TP>(g, i, ox)) p.cell[n] = -1;
    }
}

}  // namespace pic
