// boris_tile.cuh -- fused gather + Boris push + zigzag deposit, one CTA per
// tile of cells (the whole-step path of the explicit Buneman/Tristan solver).
//
// Particles are ordered by a tile-major cell key (sort.cuh), so tile t owns
// the contiguous range [off[t*T3], off[(t+1)*T3]).  A CTA
//   1. stages the six Yee components of the tile plus one cell of halo in
//      shared memory (the gather of a particle in cell c reads nodes c, c+1
//      and cell centres c-1..c+1),
//   2. pushes every particle of the tile, gathering from shared memory, and
//      accumulates its 24 zigzag current terms into a shared-memory current
//      block covering the tile plus two cells of halo (a particle moves at
//      most one cell per step; the zigzag touches new cell -1 .. +2),
//   3. writes that block, unreduced, to a per-tile partial buffer.
// k_assemble_j then sums the (up to 27) partials of every cell in a fixed
// order into the FP64 current grid: no global floating-point atomics.
// A particle that has drifted out of its tile since the last sort (or that
// moves more than one cell) takes the global path: global gather and FP64
// global atomics into a separate correction grid.
#pragma once
#include "boris.cuh"
#include "types.cuh"

namespace pic {

constexpr int kTileThreads = 256;
template <typename TP, typename TF>
__global__ void __launch_bounds__(kTileThreads) k_push_deposit_tile(GridP g, TileGeom t, TileShape s, SpeciesSet<TP> S,
                                                                    const TF* __restrict__ E, const TF* __restrict__ B,
                                                                    TP* __restrict__ Jpart, double* __restrict__ Jfix) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int F = s.fx * s.fy * s.fz;
    TF* sF = reinterpret_cast<TF*>(smem_raw);                 // 6 * F
    TP* sJ = reinterpret_cast<TP*>(smem_raw + ((6 * F * sizeof(TF) + 15) & ~size_t(15)));   // 3 * jcells
    const long long JC = s.jcells;
    const int ntiles = t.ntx * t.nty * t.ntz;
    const int T3 = t.tx * t.ty * t.tz;
    const long long N = g.N;
    const TP dt = TP(g.dt);
    const TP idx = TP(1.0 / g.dx), idy = TP(1.0 / g.dy), idz = TP(1.0 / g.dz);
    const TP vol = TP(g.dx) * TP(g.dy) * TP(g.dz);

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int ti = tile % t.ntx, tj = (tile / t.ntx) % t.nty, tk = tile / (t.ntx * t.nty);
        const int lox = ti * t.tx, loy = tj * t.ty, loz = tk * t.tz;
        // 1. stage fields
        for (int e = threadIdx.x; e < F; e += blockDim.x) {
            int a = e % s.fx, b = (e / s.fx) % s.fy, c = e / (s.fx * s.fy);
            long long gi = linw(g, lox - s.hx + a, loy - s.hy + b, loz - s.hz + c);
#pragma unroll
            for (int comp = 0; comp < 3; ++comp) {
                sF[comp * F + e] = E[comp * N + gi];
                sF[(3 + comp) * F + e] = B[comp * N + gi];
            }
        }
        for (long long e = threadIdx.x; e < 3 * JC; e += blockDim.x) sJ[e] = TP(0);
        __syncthreads();

        // 2. particles of every species in this tile
        for (int sp = 0; sp < S.ns; ++sp) {
            const PartView<TP> P = S.p[sp];
            const TP q = S.q[sp], m = S.m[sp];
            const TP beta = q * dt / (TP(2) * m);
            const TP fcd = q * S.w[sp] / vol;
            const long long pb = S.off[sp][(long long)tile * T3], pe = S.off[sp][(long long)(tile + 1) * T3];
            for (long long base = pb; base < pe; base += kTileThreads) {
                // spread consecutive lanes over the chunk so that lanes of a
                // warp hit different cells in the shared-memory atomics
                const int tid = threadIdx.x;
                const long long n = base + (tid & 31) * (kTileThreads / 32) + (tid >> 5);
                if (n >= pe) continue;
                int cell = P.cell[n];
                TP ox = P.ox[n], oy = P.oy[n], oz = P.oz[n];
                int i, j, k;
                decode(g, cell, i, j, k);
                const int li = i - lox, lj = j - loy, lk = k - loz;
                const bool inside = (li >= 0 && li < t.tx && lj >= 0 && lj < t.ty && lk >= 0 && lk < t.tz);
                TP e3[3], b3[3];
                if (inside) {
                    // staged gather (correlation.cpp:441-600 with local indices)
                    int nX[2], cX[2], nY[2], cY[2], nZ[2], cZ[2];
                    TP wnX[2], wcX[2], wnY[2], wcY[2], wnZ[2], wcZ[2];
                    node_w(ox, li + s.hx, 1 << 30, nX, wnX); cell_w(ox, li + s.hx, 1 << 30, cX, wcX);
                    if (g.y3) { node_w(oy, lj + s.hy, 1 << 30, nY, wnY); cell_w(oy, lj + s.hy, 1 << 30, cY, wcY); }
                    else { node_w(oy, 0, 1, nY, wnY); cell_w(oy, 0, 1, cY, wcY); }
                    if (g.z3) { node_w(oz, lk + s.hz, 1 << 30, nZ, wnZ); cell_w(oz, lk + s.hz, 1 << 30, cZ, wcZ); }
                    else { node_w(oz, 0, 1, nZ, wnZ); cell_w(oz, 0, 1, cZ, wcZ); }
                    e3[0] = e3[1] = e3[2] = TP(0); b3[0] = b3[1] = b3[2] = TP(0);
                    auto L = [&](int a, int b, int c) { return (c * s.fy + b) * s.fx + a; };
#pragma unroll
                    for (int a = 0; a < 2; ++a)
#pragma unroll
                        for (int bb = 0; bb < 2; ++bb)
#pragma unroll
                            for (int cc = 0; cc < 2; ++cc) {
                                e3[0] += TP(sF[0 * F + L(cX[a], nY[bb], nZ[cc])]) * wcX[a] * wnY[bb] * wnZ[cc];
                                e3[1] += TP(sF[1 * F + L(nX[a], cY[bb], nZ[cc])]) * wnX[a] * wcY[bb] * wnZ[cc];
                                e3[2] += TP(sF[2 * F + L(nX[a], nY[bb], cZ[cc])]) * wnX[a] * wnY[bb] * wcZ[cc];
                                b3[0] += TP(sF[3 * F + L(nX[a], cY[bb], cZ[cc])]) * wnX[a] * wcY[bb] * wcZ[cc];
                                b3[1] += TP(sF[4 * F + L(cX[a], nY[bb], cZ[cc])]) * wcX[a] * wnY[bb] * wcZ[cc];
                                b3[2] += TP(sF[5 * F + L(cX[a], cY[bb], nZ[cc])]) * wcX[a] * wcY[bb] * wnZ[cc];
                            }
                } else {
                    yee_gather<TP, TF>(g, cell, ox, oy, oz, E, B, e3, b3);
                }
                TP mom[3] = {P.px[n], P.py[n], P.pz[n]};
                boris<TP>(q, m, dt, beta, e3, b3, mom);
                P.px[n] = mom[0]; P.py[n] = mom[1]; P.pz[n] = mom[2];
                TP v[3];
                velocity<TP>(mom, m, v);
                int ni = i, nj = j, nk = k;
                advance_axis<TP>(ox, ni, (v[0] * dt) * idx, g.nx);
                advance_axis<TP>(oy, nj, (v[1] * dt) * idy, g.ny);
                advance_axis<TP>(oz, nk, (v[2] * dt) * idz, g.nz);
                P.ox[n] = ox; P.oy[n] = oy; P.oz[n] = oz;
                P.cell[n] = (int)lin(g, ni, nj, nk);
                // unwrapped shift of the new cell relative to the old one
                auto shift = [](int nw, int old, int nn) {
                    int d = nw - old;
                    if (d > nn / 2) d -= nn;
                    if (d < -nn / 2) d += nn;
                    return d;
                };
                const int sx = shift(ni, i, g.nx), sy = shift(nj, j, g.ny), sz = shift(nk, k, g.nz);
                const bool local_dep = inside && sx >= -1 && sx <= 1 && sy >= -1 && sy <= 1 && sz >= -1 && sz <= 1;
                if (local_dep) {
                    const int bx = li + s.gx + sx, by = (g.y3 ? lj + sy : 0) + s.gy, bz = (g.z3 ? lk + sz : 0) + s.gz;
                    zigzag_terms<TP>(g, fcd, ox, oy, oz, v, [&](int comp, int di, int dj, int dk, TP val) {
                        int a = bx + di, b = by + dj, c = bz + dk;
                        if (a >= 0 && a < s.jx && b >= 0 && b < s.jy && c >= 0 && c < s.jz)
                            atomicAdd(&sJ[comp * JC + ((long long)c * s.jy + b) * s.jx + a], val);
                        else
                            atomicAdd(&Jfix[comp * N + linw(g, ni + di, nj + dj, nk + dk)], double(val));
                    });
                } else {
                    zigzag_terms<TP>(g, fcd, ox, oy, oz, v, [&](int comp, int di, int dj, int dk, TP val) {
                        atomicAdd(&Jfix[comp * N + linw(g, ni + di, nj + dj, nk + dk)], double(val));
                    });
                }
            }
        }
        __syncthreads();
        // 3. unreduced tile partials, coalesced
        TP* dst = Jpart + (long long)tile * 3 * JC;
        for (long long e = threadIdx.x; e < 3 * JC; e += blockDim.x) dst[e] = sJ[e];
        __syncthreads();
    }
}

// J[c] = Jfix[c] + sum of every tile partial that covers cell c, tiles and
// periodic images visited in a fixed order (deterministic, FP64).
template <typename TP>
__global__ void __launch_bounds__(256) k_assemble_j(GridP g, TileGeom t, TileShape s, const TP* __restrict__ Jpart,
                                                    const double* __restrict__ Jfix, double* __restrict__ J) {
    const long long JC = s.jcells;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.N;
         c += (long long)gridDim.x * blockDim.x) {
        int p[3];
        decode(g, (int)c, p[0], p[1], p[2]);
        const int n[3] = {g.nx, g.ny, g.nz};
        const int te[3] = {t.tx, t.ty, t.tz};
        const int nt[3] = {t.ntx, t.nty, t.ntz};
        const int je[3] = {s.jx, s.jy, s.jz};
        const int hg[3] = {s.gx, s.gy, s.gz};
        // per axis: every (tile, local index) whose current block holds this
        // cell or one of its periodic images, in increasing image order
        constexpr int kCand = 16;
        int cand_t[3][kCand], cand_l[3][kCand], cnt[3];
        for (int ax = 0; ax < 3; ++ax) {
            cnt[ax] = 0;
            for (int sh = -1; sh <= 1; ++sh) {
                const int q = p[ax] + sh * n[ax];
                // block of tile T spans [T*te - hg, T*te - hg + je)
                int tlo = q + hg[ax] - je[ax] + 1;
                tlo = tlo >= 0 ? (tlo + te[ax] - 1) / te[ax] : -((-tlo) / te[ax]);
                int thi = q + hg[ax];
                thi = thi >= 0 ? thi / te[ax] : -((-thi + te[ax] - 1) / te[ax]);
                if (tlo < 0) tlo = 0;
                if (thi > nt[ax] - 1) thi = nt[ax] - 1;
                for (int T = tlo; T <= thi && cnt[ax] < kCand; ++T) {
                    cand_t[ax][cnt[ax]] = T;
                    cand_l[ax][cnt[ax]] = q - (T * te[ax] - hg[ax]);
                    cnt[ax]++;
                }
            }
        }
        double acc[3] = {Jfix[c], Jfix[g.N + c], Jfix[2 * g.N + c]};
        for (int a = 0; a < cnt[0]; ++a)
            for (int b = 0; b < cnt[1]; ++b)
                for (int d = 0; d < cnt[2]; ++d) {
                    long long tile = ((long long)cand_t[2][d] * t.nty + cand_t[1][b]) * t.ntx + cand_t[0][a];
                    long long e = ((long long)cand_l[2][d] * s.jy + cand_l[1][b]) * s.jx + cand_l[0][a];
                    const TP* src = Jpart + tile * 3 * JC;
                    acc[0] += double(src[e]);
                    acc[1] += double(src[JC + e]);
                    acc[2] += double(src[2 * JC + e]);
                }
        J[c] = acc[0]; J[g.N + c] = acc[1]; J[2 * g.N + c] = acc[2];
    }
}

}  // namespace pic
