// implicit_tile.cuh -- moment deposition of the implicit path over tiles of
// cells (updateElectroMagneticParameters, PIC++/momentum_collecting.cpp
// 365-584, with the pressure tensor at the particle's own cells).
//
// Particles are ordered by the tile-major cell key (sort.cuh).  One CTA owns
// a tile and accumulates, in shared memory,
//   * on nodes (tile + h halo + 1):  J-hat (3) and mu (9), 8 nodes/particle;
//   * on cells (tile + h halo + 2):  rho-hat (1) and Pi (6 of the symmetric
//     9), 8 of the 27 cells around the particle's cell.
// A warp takes one cell key at a time and walks its particles 32 at a time.
// Lanes holding the same (current) cell share one stencil base, so their
// 96 node and 189 cell products (27 slots, zero weight outside the
// particle's octant) are summed with a butterfly transpose-reduction: after
// five exchange rounds lane L holds the warp total of product L of a
// 32-product pass, and adds it to shared memory with one atomic.  Runs of
// only a few lanes add their products directly; particles more than h cells
// outside the tile add theirs to the FP64 grids with global atomics.  The
// tile's block is finally added to the FP64 grids (global atomics only on
// block entries, 22 per node/cell).
#pragma once
#include "implicit_particles.cuh"

namespace pic {

constexpr int kImpThreads = 256;
constexpr int kXposeMin = 4;   // fewest lanes of one cell that take the transpose-reduction

// Symmetric pressure components kept in shared memory, q = 0..5:
// (a, b) = (0,0) (0,1) (0,2) (1,1) (1,2) (2,2).
__host__ __device__ constexpr int sym_a(int q) { return q < 3 ? 0 : (q < 5 ? 1 : 2); }
__host__ __device__ constexpr int sym_b(int q) { return q < 3 ? q : (q < 5 ? q - 2 : 2); }

// Butterfly transpose-reduction of one 32-product pass: returns, in lane L,
// the sum over the warp of v[L].
template <typename A>
__device__ __forceinline__ A xpose_sum(A v[32], int lane) {
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const bool up = (lane & w) != 0;
#pragma unroll
        for (int i = 0; i < w; ++i) {
            const A send = up ? v[i] : v[i + w];
            const A keep = up ? v[i + w] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, w);
        }
    }
    return v[0];
}

// Node / cell weights of one axis (node_w and cell_w of common.cuh, in the
// three-slot form c-1, c, c+1 for cells).
template <typename T>
__device__ __forceinline__ void axis_weights(T u, bool act, T wn[2], T wc[3]) {
    if (!act) { wn[0] = T(1); wn[1] = T(0); wc[0] = T(0); wc[1] = T(1); wc[2] = T(0); return; }
    if (u < T(0.5)) { wn[0] = T(0.5) + (T(0.5) - u); wn[1] = T(1) - wn[0]; }
    else            { wn[1] = T(0.5) + (u - T(0.5)); wn[0] = T(1) - wn[1]; }
    if (u < T(0.5)) { wc[1] = T(0.5) + u; wc[0] = T(1) - wc[1]; wc[2] = T(0); }
    else            { wc[1] = T(0.5) + (T(1) - u); wc[2] = T(1) - wc[1]; wc[0] = T(0); }
}

// Local index of global cell index c on an axis of n cells relative to a
// tile starting at x0, chosen within [-h, t - 1 + h] when a periodic image
// lies there; false if none does.
__device__ __forceinline__ bool local_axis(int c, int x0, int t, int h, int n, int& l) {
    l = c - x0;
    if (l >= -h && l <= t - 1 + h) return true;
    if (l - n >= -h && l - n <= t - 1 + h) { l -= n; return true; }
    if (l + n >= -h && l + n <= t - 1 + h) { l += n; return true; }
    return false;
}

// All 8 node and 8 cell contributions of one particle to the FP64 grids
// (particles outside the tile's block; rare).
template <typename T>
__device__ __noinline__ void imp_deposit_global(const GridP& g, int i, int j, int k, T ox, T oy, T oz,
                                                const double* QN, const double* QC, double* __restrict__ J,
                                                double* __restrict__ mu, double* __restrict__ rho,
                                                double* __restrict__ Pi) {
    int X[2], Y[2], Z[2];
    T wx[2], wy[2], wz[2];
    node_w(ox, i, g.nx, X, wx); node_w(oy, j, g.ny, Y, wy); node_w(oz, k, g.nz, Z, wz);
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
                double wgt = double(wx[a]) * double(wy[b]) * double(wz[c]);
                if (wgt == 0.0) continue;
                long long id = lin(g, X[a], Y[b], Z[c]);
                for (int d = 0; d < 3; ++d) atomicAdd(&J[d * g.N + id], QN[d] * wgt);
                for (int d = 0; d < 9; ++d) atomicAdd(&mu[d * g.N + id], QN[3 + d] * wgt);
            }
    cell_w(ox, i, g.nx, X, wx); cell_w(oy, j, g.ny, Y, wy); cell_w(oz, k, g.nz, Z, wz);
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
                double wgt = double(wx[a]) * double(wy[b]) * double(wz[c]);
                if (wgt == 0.0) continue;
                long long id = lin(g, X[a], Y[b], Z[c]);
                atomicAdd(&rho[id], QC[0] * wgt);
                for (int s = 0; s < 6; ++s) {
                    double v = QC[1 + s] * wgt;
                    atomicAdd(&Pi[(3 * sym_a(s) + sym_b(s)) * g.N + id], v);
                    if (sym_a(s) != sym_b(s)) atomicAdd(&Pi[(3 * sym_b(s) + sym_a(s)) * g.N + id], v);
                }
            }
}

template <typename T, typename A>
__global__ void __launch_bounds__(kImpThreads, 2) k_implicit_deposit_tile(GridP g, TileGeom t, ImpBlock bk,
                                                                       ImpSpecies<T> S, const double* __restrict__ E,
                                                                       const double* __restrict__ B,
                                                                       double* __restrict__ J, double* __restrict__ mu,
                                                                       double* __restrict__ rho,
                                                                       double* __restrict__ Pi) {
    extern __shared__ __align__(16) unsigned char imp_smem[];
    A* sN = reinterpret_cast<A*>(imp_smem);   // [12][NB]
    A* sC = sN + 12 * bk.NB;                  // [7][CB]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int T3 = t.tx * t.ty * t.tz;
    const int ntiles = t.ntx * t.nty * t.ntz;
    const double PI_D = 3.14159265358979323846;
    const double ivol = 1.0 / (g.dx * g.dy * g.dz);
    const bool ax = g.nx > 1, ay = g.y3, az = g.z3;
    const int hx = ax ? bk.h : 0, hy = ay ? bk.h : 0, hz = az ? bk.h : 0;
    const int nsy = bk.nbx, nsz = bk.nbx * bk.nby;
    const int csy = bk.cbx, csz = bk.cbx * bk.cby;
    const int oxn = ax ? 1 : 0, oyn = ay ? nsy : 0, ozn = az ? nsz : 0;   // corner strides
    const int oxc = ax ? 1 : 0, oyc = ay ? csy : 0, ozc = az ? csz : 0;   // slot strides
    const int tot = 12 * bk.NB + 7 * bk.CB;

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int ti = tile % t.ntx, tj = (tile / t.ntx) % t.nty, tk = tile / (t.ntx * t.nty);
        const int x0 = ti * t.tx, y0 = tj * t.ty, z0 = tk * t.tz;
        for (int e = threadIdx.x; e < tot; e += blockDim.x) sN[e] = A(0);
        __syncthreads();
        for (int s = 0; s < S.ns; ++s) {
            const PartView<T> p = S.p[s];
            const int* __restrict__ off = S.off[s];
            const double qs = S.q[s], ms = S.m[s], ws = S.w[s];
            const T beta = T(0.5 * qs * g.dt / ms);
            const double cq = qs * ws * ivol;
            const double cm = -(ws * g.theta * g.dt * g.dt * 2 * PI_D * qs * qs / ms) * ivol;
            for (int lc = warp; lc < T3; lc += nwarps) {
                const int kk = tile * T3 + lc;
                const int b0 = off[kk], b1 = off[kk + 1];
                for (int c0 = b0; c0 < b1; c0 += 32) {
                    const int n = c0 + lane;
                    const bool valid = n < b1;
                    A QN[12], QC[7], wn[8], wc[27];
                    int cell = -1, nb = 0, cb = 0;
                    bool inb = false;
                    if (valid) {
                        cell = p.cell[n];
                        int i, j, k;
                        decode(g, cell, i, j, k);
                        const T ox = p.ox[n], oy = p.oy[n], oz = p.oz[n];
                        T mom[3] = {p.px[n], p.py[n], p.pz[n]};
                        T gam, v[3];
                        gamma_vel<T>(mom, T(ms), gam, v);
                        T e[3], bf[3];
                        gather_node<T>(g, i, j, k, ox, oy, oz, E, e);
                        gather_cell<T>(g, i, j, k, ox, oy, oz, B, bf);
                        T al[9];
                        alpha_tensor<T>(beta, v, gam, e, bf, al);
                        const T vg[3] = {v[0] * gam, v[1] * gam, v[2] * gam};
                        A rv[3];
#pragma unroll
                        for (int a = 0; a < 3; ++a)
                            rv[a] = A(al[3 * a] * vg[0] + al[3 * a + 1] * vg[1] + al[3 * a + 2] * vg[2]);
#pragma unroll
                        for (int d = 0; d < 3; ++d) QN[d] = rv[d] * A(cq);
#pragma unroll
                        for (int d = 0; d < 9; ++d) QN[3 + d] = A(al[d]) * A(cm);
                        QC[0] = A(cq);
#pragma unroll
                        for (int q = 0; q < 6; ++q) QC[1 + q] = A(cq) * (rv[sym_a(q)] * rv[sym_b(q)]);
                        T nwx[2], nwy[2], nwz[2], cwx[3], cwy[3], cwz[3];
                        axis_weights<T>(ox, ax, nwx, cwx);
                        axis_weights<T>(oy, ay, nwy, cwy);
                        axis_weights<T>(oz, az, nwz, cwz);
#pragma unroll
                        for (int c = 0; c < 8; ++c) wn[c] = A(nwx[c & 1] * nwy[(c >> 1) & 1] * nwz[c >> 2]);
#pragma unroll
                        for (int q = 0; q < 27; ++q) wc[q] = A(cwx[q % 3] * cwy[(q / 3) % 3] * cwz[q / 9]);
                        int li = 0, lj = 0, lk = 0;
                        inb = local_axis(i, x0, t.tx, hx, g.nx, li) && local_axis(j, y0, t.ty, hy, g.ny, lj) &&
                              local_axis(k, z0, t.tz, hz, g.nz, lk);
                        if (inb) {
                            nb = (lk + hz) * nsz + (lj + hy) * nsy + (li + hx);
                            cb = (lk + hz) * csz + (lj + hy) * csy + (li + hx);
                        } else {
                            double qn[12], qc[7];
#pragma unroll
                            for (int d = 0; d < 12; ++d) qn[d] = double(QN[d]);
#pragma unroll
                            for (int d = 0; d < 7; ++d) qc[d] = double(QC[d]);
                            imp_deposit_global<T>(g, i, j, k, ox, oy, oz, qn, qc, J, mu, rho, Pi);
                        }
                    }
                    unsigned pending = __ballot_sync(0xffffffffu, valid && inb);
                    while (pending) {
                        const int leader = __ffs(pending) - 1;
                        const int lcell = __shfl_sync(0xffffffffu, cell, leader);
                        const bool me = ((pending >> lane) & 1u) && cell == lcell;
                        const unsigned mem = __ballot_sync(0xffffffffu, me);
                        pending &= ~mem;
                        if (__popc(mem) >= kXposeMin) {
                            const int nbL = __shfl_sync(0xffffffffu, nb, leader);
                            const int cbL = __shfl_sync(0xffffffffu, cb, leader);
                            A v[32];
#pragma unroll
                            for (int r = 0; r < 3; ++r) {
#pragma unroll
                                for (int x = 0; x < 32; ++x) v[x] = me ? QN[4 * r + x / 8] * wn[x % 8] : A(0);
                                const A sum = xpose_sum<A>(v, lane);
                                const int q = 4 * r + lane / 8, c = lane % 8;
                                if (sum != A(0))
                                    atomicAdd(&sN[q * bk.NB + nbL + (c & 1) * oxn + ((c >> 1) & 1) * oyn + (c >> 2) * ozn],
                                              sum);
                            }
#pragma unroll
                            for (int r = 0; r < 6; ++r) {
#pragma unroll
                                for (int x = 0; x < 32; ++x) {
                                    const int idx = 32 * r + x;
                                    v[x] = (idx < 189 && me) ? QC[idx / 27] * wc[idx % 27] : A(0);
                                }
                                const A sum = xpose_sum<A>(v, lane);
                                const int idx = 32 * r + lane;
                                if (idx < 189 && sum != A(0)) {
                                    const int q = idx / 27, sl = idx % 27;
                                    atomicAdd(&sC[q * bk.CB + cbL + (sl % 3) * oxc + ((sl / 3) % 3) * oyc + (sl / 9) * ozc],
                                              sum);
                                }
                            }
                        } else if (me) {
#pragma unroll
                            for (int c = 0; c < 8; ++c) {
                                if (wn[c] == A(0)) continue;
                                const int o = nb + (c & 1) * oxn + ((c >> 1) & 1) * oyn + (c >> 2) * ozn;
#pragma unroll
                                for (int q = 0; q < 12; ++q) atomicAdd(&sN[q * bk.NB + o], QN[q] * wn[c]);
                            }
#pragma unroll
                            for (int sl = 0; sl < 27; ++sl) {
                                if (wc[sl] == A(0)) continue;
                                const int o = cb + (sl % 3) * oxc + ((sl / 3) % 3) * oyc + (sl / 9) * ozc;
#pragma unroll
                                for (int q = 0; q < 7; ++q) atomicAdd(&sC[q * bk.CB + o], QC[q] * wc[sl]);
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();
        // flush the block into the FP64 grids
        for (int e = threadIdx.x; e < bk.NB; e += blockDim.x) {
            const int lx = e % bk.nbx, ly = (e / bk.nbx) % bk.nby, lz = e / (bk.nbx * bk.nby);
            const long long id = linw(g, x0 - hx + lx, y0 - hy + ly, z0 - hz + lz);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const A v = sN[d * bk.NB + e];
                if (v != A(0)) atomicAdd(&J[d * g.N + id], double(v));
            }
#pragma unroll
            for (int d = 0; d < 9; ++d) {
                const A v = sN[(3 + d) * bk.NB + e];
                if (v != A(0)) atomicAdd(&mu[d * g.N + id], double(v));
            }
        }
        for (int e = threadIdx.x; e < bk.CB; e += blockDim.x) {
            const int lx = e % bk.cbx, ly = (e / bk.cbx) % bk.cby, lz = e / (bk.cbx * bk.cby);
            const long long id = linw(g, x0 - hx - (ax ? 1 : 0) + lx, y0 - hy - (ay ? 1 : 0) + ly,
                                      z0 - hz - (az ? 1 : 0) + lz);
            const A r = sC[e];
            if (r != A(0)) atomicAdd(&rho[id], double(r));
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const A v = sC[(1 + q) * bk.CB + e];
                if (v == A(0)) continue;
                atomicAdd(&Pi[(3 * sym_a(q) + sym_b(q)) * g.N + id], double(v));
                if (sym_a(q) != sym_b(q)) atomicAdd(&Pi[(3 * sym_b(q) + sym_a(q)) * g.N + id], double(v));
            }
        }
        __syncthreads();
    }
}

}  // namespace pic
