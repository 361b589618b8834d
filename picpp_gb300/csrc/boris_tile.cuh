// boris_tile.cuh -- fused gather + Boris push + zigzag deposit, one CTA per
// tile of cells (the whole-step path of the explicit Buneman/Tristan solver).
//
// Particles are ordered by a tile-major cell key (sort.cuh), so tile t owns
// the contiguous range [off[t*T3], off[(t+1)*T3]) of every species.  A CTA
//   1. stages the six Yee components of the tile plus two cells of halo in
//      shared memory: the gather of a particle in cell c reads nodes c, c+1
//      and cell centres c-1..c+1, so particles up to one cell outside their
//      tile (drift since the last sort) still gather from shared memory;
//   2. walks the tile's particles in chunks of 32 consecutive particles per
//      warp (coalesced loads and stores) and pushes them.  The zigzag current
//      of a particle is two segments, each with 12 terms at fixed positions
//      relative to one cell: the segment from the old position to the relay
//      point (in the old cell) and the one from the relay point to the new
//      position (in the new cell).  Lanes holding the same cell (particles
//      are sorted by cell) sum each segment's 12 values with a segmented
//      shuffle reduction, and the run totals go into a shared-memory current
//      block (tile plus two cells of halo).  FP32 particles: the block is
//      exact 64-bit fixed point in two 32-bit words per entry, added with
//      native 32-bit integer shared atomics (FP32 shared atomics are
//      compare-and-swap loops that collapse under address conflicts), the
//      adds of a warp's run heads spread over its lanes; the block sums are
//      exact and order-independent.  FP64 particles: FP64 shared atomics.
//      Each warp copies its next chunk of particles into shared memory with
//      cp.async while it pushes the current one;
//   3. writes the block, unreduced, to a per-tile partial buffer (for FP32
//      particles the exact fixed-point sums as 64-bit integers).
// k_assemble_j then sums the partials of every cell in a fixed order into
// the FP64 current grid (FP32 particles: exact integer sums, scaled once):
// no global floating-point atomics on the fast path.
// A particle more than one cell outside its tile, or whose zigzag segments
// leave the tile's current block, is left to k_push_deposit_deferred: the
// fused kernel sets its bit in a per-species mask and the deferred pass
// pushes it with the global gather and/or deposits its current with FP64
// global atomics into a correction grid.  The fused kernel itself calls no
// function out of line (a call site costs its hot loop register spills).
#pragma once
#include "boris.cuh"
#include "types.cuh"

namespace pic {

#ifndef PIC_TILE_THREADS
#define PIC_TILE_THREADS 512   // threads per CTA of the fused explicit kernel (64 registers at 2 CTAs/SM)
#endif
constexpr int kTileThreads = PIC_TILE_THREADS;
#ifndef PIC_TILE_MIN_BLOCKS
#define PIC_TILE_MIN_BLOCKS 2   // CTAs per SM the register budget is sized for
#endif

template <typename TP>
__device__ __forceinline__ TP lerp(TP a, TP b, TP w) { return a + w * (b - a); }

// Trilinear value of one staggered component from the staged block: base is
// the block index of the lower corner, sy/sz the strides, (wx, wy, wz) the
// weights of the upper corner.
template <typename TP, typename TF>
__device__ __forceinline__ TP tri(const TF* __restrict__ F, int base, int sy, int sz, TP wx, TP wy, TP wz) {
    TP v000 = TP(F[base]), v100 = TP(F[base + 1]);
    TP v010 = TP(F[base + sy]), v110 = TP(F[base + sy + 1]);
    TP v001 = TP(F[base + sz]), v101 = TP(F[base + sz + 1]);
    TP v011 = TP(F[base + sy + sz]), v111 = TP(F[base + sy + sz + 1]);
    TP a = lerp(lerp(v000, v100, wx), lerp(v010, v110, wx), wy);
    TP b = lerp(lerp(v001, v101, wx), lerp(v011, v111, wx), wy);
    return lerp(a, b, wz);
}

// The 24 zigzag terms of a particle straight into the FP64 correction grid.
template <typename TP>
__device__ __forceinline__ void deposit_global(const GridP& g, TP fcd, TP ox, TP oy, TP oz, const TP v[3], int ni,
                                               int nj, int nk, double* __restrict__ Jfix) {
    zigzag_terms<TP>(g, fcd, ox, oy, oz, v, [&](int comp, int di, int dj, int dk, TP val) {
        atomicAdd(&Jfix[comp * g.N + linw(g, ni + di, nj + dj, nk + dk)], double(val));
    }, g.wall && ni == kTristanWallNode);
}

// Sets the bits of a warp's chunk of particles s0 .. s0 + 31 (bit l for
// particle s0 + l) in a particle bit mask.
__device__ __forceinline__ void set_defer_bits(unsigned* __restrict__ mask, long long s0, unsigned bits) {
    if (!bits) return;
    const long long w = s0 >> 5;
    const int sh = (int)(s0 & 31);
    atomicOr(&mask[w], bits << sh);
    if (sh && (bits >> (32 - sh))) atomicOr(&mask[w + 1], bits >> (32 - sh));
}

// One zigzag segment's 12 terms relative to its cell
// (momentum_collecting.cpp:200-230): Jx at (c, j+dj, k+dk) -> slot 2dk+dj,
// Jy at (i+di, c, k+dk) -> 4+2dk+di, Jz at (i+di, j+dj, c) -> 8+2dj+di.
template <typename TP>
__device__ __forceinline__ void segment_slots(TP Fx, TP Fy, TP Fz, TP Wx, TP Wy, TP Wz, TP a[12]) {
    const TP ux = TP(1) - Wx, uy = TP(1) - Wy, uz = TP(1) - Wz;
    a[0] = Fx * uy * uz; a[1] = Fx * Wy * uz; a[2] = Fx * uy * Wz; a[3] = Fx * Wy * Wz;
    a[4] = Fy * ux * uz; a[5] = Fy * Wx * uz; a[6] = Fy * ux * Wz; a[7] = Fy * Wx * Wz;
    a[8] = Fz * ux * uy; a[9] = Fz * Wx * uy; a[10] = Fz * ux * Wy; a[11] = Fz * Wx * Wy;
}

// Segmented sum of a[] over runs of lanes with equal key; returns true in the
// first lane of each run, which then holds the run's totals.
template <typename TP>
__device__ __forceinline__ bool run_sum(int key, TP a[12]) {
    const int lane = threadIdx.x & 31;
    const int prev = __shfl_up_sync(0xffffffffu, key, 1);
    const bool head = lane == 0 || key != prev;
    const unsigned H = __ballot_sync(0xffffffffu, head);
    if (H != 0xffffffffu) {
        const unsigned after = H & ~((2u << lane) - 1u);
        const int seg_end = after ? (__ffs(after) - 2) : 31;
        // only as many doubling rounds as the longest run needs
        const unsigned run = __reduce_max_sync(0xffffffffu, head ? (unsigned)(seg_end - lane + 1) : 1u);
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            if ((unsigned)d >= run) break;
            const bool take = lane + d <= seg_end;
#pragma unroll
            for (int q = 0; q < 12; ++q) {
                TP o = __shfl_down_sync(0xffffffffu, a[q], d);
                if (take) a[q] += o;
            }
        }
    }
    return head;
}

// Adds one run's 12 totals at block cell c (strides X0, XY).
template <typename TP>
__device__ __forceinline__ void add_slots(TP* __restrict__ sJ, long long JC, int c, int X0, int XY, int ey, int ez,
                                          const TP a[12]) {
    TP* jx = sJ;
    TP* jy = sJ + JC;
    TP* jz = sJ + 2 * JC;
    atomicAdd(&jx[c], a[0]);
    if (ey) atomicAdd(&jx[c + X0], a[1]);
    if (ez) atomicAdd(&jx[c + XY], a[2]);
    if (ey && ez) atomicAdd(&jx[c + X0 + XY], a[3]);
    atomicAdd(&jy[c], a[4]);
    atomicAdd(&jy[c + 1], a[5]);
    if (ez) atomicAdd(&jy[c + XY], a[6]);
    if (ez) atomicAdd(&jy[c + 1 + XY], a[7]);
    atomicAdd(&jz[c], a[8]);
    atomicAdd(&jz[c + 1], a[9]);
    if (ey) atomicAdd(&jz[c + X0], a[10]);
    if (ey) atomicAdd(&jz[c + 1 + X0], a[11]);
}

// Fixed-point current block of the FP32 path: a run total a becomes the
// integer x = rint(a * sc) (sc a power of two with |x| < 2^40), and the block
// holds each entry as a 64-bit two's-complement sum in a low (unsigned) and a
// high (signed) 32-bit word, the low word's carry added to the high one.
// Shared 32-bit integer atomics are native; the sums are exact and
// independent of the order of the adds.  The split uses 32-bit conversions
// and integer operations only (64-bit integer conversions run on the FP64
// pipe, which is slow on this GPU): |x| = h 2^31 + l with h < 2^9, l < 2^31.
__device__ __forceinline__ void fx_add(unsigned* __restrict__ lo, int* __restrict__ hi, int e, float xf) {
    const float m = fabsf(xf);
    const float hf = floorf(m * 4.656612873077393e-10f);            // m / 2^31, exact power-of-two scaling
    const unsigned h = (unsigned)hf;
    const unsigned l = __float2uint_rn(m - hf * 2147483648.0f);      // exact remainder, rounded to an integer
    const unsigned al = ((h & 1u) << 31) | l;                        // |x| in base 2^32
    const unsigned ah = h >> 1;
    // two's complement of the 64-bit value for x < 0, without branches (a
    // zero x adds nothing)
    const unsigned sg = xf < 0.f ? 0xffffffffu : 0u;
    const unsigned xl = (al ^ sg) - sg;
    const unsigned xh = (ah ^ sg) + (sg & (xl == 0u ? 1u : 0u));
    const unsigned old = atomicAdd(&lo[e], xl);
    const unsigned carry = (old + xl < old) ? 1u : 0u;
    atomicAdd(&hi[e], (int)(xh + carry));
}

// add_slots in fixed point.
// 32-bit offsets: a block holds 3 x (tile + 4)^3 entries at most.
__device__ __forceinline__ void add_slots_fx(unsigned* __restrict__ lo, int* __restrict__ hi, int JC, int c,
                                             int X0, int XY, int ey, int ez, const float a[12], float sc) {
    const int off[12] = {c, c + X0, c + XY, c + X0 + XY,
                               JC + c, JC + c + 1, JC + c + XY, JC + c + 1 + XY,
                               2 * JC + c, 2 * JC + c + 1, 2 * JC + c + X0, 2 * JC + c + 1 + X0};
    const bool use[12] = {true, ey != 0, ez != 0, ey && ez, true, true, ez != 0, ez != 0, true, true, ey != 0, ey != 0};
#pragma unroll
    for (int q = 0; q < 12; ++q)
        if (use[q]) fx_add(lo, hi, off[q], a[q] * sc);
}

// Run heads whose totals one warp spreads over its lanes, and the per-warp
// shared scratch that holds them (12 totals and the block cell of each head,
// 16-byte aligned).
constexpr int kSpreadHeads = 10;
constexpr int kSpreadBytes = (kSpreadHeads * 12 * 4 + kSpreadHeads * 4 + 15) & ~15;

// The fixed-point adds of one reduced segment: the run heads (head, key >= 0)
// hold 12 totals each.  With at most kSpreadHeads heads in the warp (the
// usual case: particles sorted by cell make runs of about the cell's
// particle count) the heads park their scaled totals in the warp's scratch
// and every lane adds about 12 heads / 32 of them, so that the conversion
// and the two atomics of each add run on all lanes instead of on the heads
// alone; with more heads each head adds its own.  Exact either way: the
// fixed-point sums do not depend on the order of the adds.
__device__ __forceinline__ void add_runs_fx(unsigned* __restrict__ lo, int* __restrict__ hi, int JC, int X0, int XY,
                                            int ey, int ez, bool head, int key, const float a[12], float sc,
                                            float* __restrict__ wv) {
    const int lane = threadIdx.x & 31;
    const bool mine = head && key >= 0;
    const unsigned H = __ballot_sync(0xffffffffu, mine);
    const int nh = __popc(H);
    if (nh > kSpreadHeads) {
        if (mine) add_slots_fx(lo, hi, JC, key, X0, XY, ey, ez, a, sc);
        return;
    }
    int* wk = reinterpret_cast<int*>(wv + kSpreadHeads * 12);
    if (mine) {
        const int o = __popc(H & ((1u << lane) - 1u));
        float4* d = reinterpret_cast<float4*>(wv + 12 * o);
        d[0] = make_float4(a[0] * sc, a[1] * sc, a[2] * sc, a[3] * sc);
        d[1] = make_float4(a[4] * sc, a[5] * sc, a[6] * sc, a[7] * sc);
        d[2] = make_float4(a[8] * sc, a[9] * sc, a[10] * sc, a[11] * sc);
        wk[o] = key;
    }
    __syncwarp();
    // value v = 12 o + q: head o, slot q of segment_slots (component q / 4;
    // bit 0 of q % 4 the first upper neighbour, bit 1 the second)
    for (int v = lane; v < 12 * nh; v += 32) {
        const int o = v / 12, q = v - 12 * o;
        const int comp = q >> 2, sub = q & 3;
        const int s1 = comp == 0 ? X0 : 1, s2 = comp == 2 ? X0 : XY;
        const bool use = ((sub & 1) == 0 || comp != 0 || ey) && ((sub & 2) == 0 || (comp == 2 ? ey : ez));
        if (use) fx_add(lo, hi, comp * JC + wk[o] + (sub & 1) * s1 + (sub >> 1) * s2, wv[v]);
    }
    __syncwarp();
}

// A warp's staged chunk of particles: cell, then ox oy oz px py pz, 32 each.
template <typename TP>
struct ChunkBuf {
    TP a[6][32];
    int cell[32];
};

// Starts the copy of particle n (this lane's slot) into the warp's buffer.
template <typename TP>
__device__ __forceinline__ void stage_particle(ChunkBuf<TP>* buf, const PartView<TP>& P, long long n, int lane) {
    cp_async<4>(&buf->cell[lane], P.cell + n);
    cp_async<sizeof(TP)>(&buf->a[0][lane], P.ox + n);
    cp_async<sizeof(TP)>(&buf->a[1][lane], P.oy + n);
    cp_async<sizeof(TP)>(&buf->a[2][lane], P.oz + n);
    cp_async<sizeof(TP)>(&buf->a[3][lane], P.px + n);
    cp_async<sizeof(TP)>(&buf->a[4][lane], P.py + n);
    cp_async<sizeof(TP)>(&buf->a[5][lane], P.pz + n);
}

// CT: compile-time tile extent of a cubic 3-D tile (8), or 0 for shapes read
// from TileShape at run time.  kWall: conductor-wall box (GridP::wall), the
// Tristan mover's reflection and escape and the zigzag wall term
// (mover.cpp:744-772, momentum_collecting.cpp:93-99); a particle that
// escaped deposits its current and is marked (cell -1) for the next sort.
template <typename TP, typename TF, int CT, bool kWall>
__global__ void __launch_bounds__(kTileThreads, PIC_TILE_MIN_BLOCKS) k_push_deposit_tile(GridP g, TileGeom t, TileShape s, SpeciesSet<TP> S,
                                                                       const TF* __restrict__ E, const TF* __restrict__ B,
                                                                       double* __restrict__ Jpart, float fx_scale,
                                                                       double inv_dt) {
    constexpr bool kFixed = sizeof(TP) == sizeof(float);   // FP32 particles: fixed-point block
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int fx = CT ? CT + 4 : s.fx, fy = CT ? CT + 4 : s.fy, fz = CT ? CT + 4 : s.fz;
    const int jx = fx, jy = fy, jz = fz;                 // both blocks: tile + 2 halo on active axes
    const int tx = CT ? CT : t.tx, ty = CT ? CT : t.ty, tz = CT ? CT : t.tz;
    const int hx = 2, hy = CT ? 2 : s.hy, hz = CT ? 2 : s.hz;
    const int F = fx * fy * fz;
    const long long JC = (long long)jx * jy * jz;
    TF* sF = reinterpret_cast<TF*>(smem_raw);   // 6 * F
    TP* sJ = reinterpret_cast<TP*>(smem_raw + ((6 * F * sizeof(TF) + 15) & ~size_t(15)));   // 3 * JC (FP64)
    unsigned* sLo = reinterpret_cast<unsigned*>(sJ);                                        // 3 * JC (FP32)
    int* sHi = reinterpret_cast<int*>(sLo + 3 * JC);                                        // 3 * JC (FP32)
    // FP32: the warps' spread scratch after the block; then every warp's
    // staged chunk of particles
    unsigned char* after_j = reinterpret_cast<unsigned char*>(sJ) + ((24 * JC + 15) & ~15ll);
    float* sW = reinterpret_cast<float*>(after_j + (threadIdx.x >> 5) * kSpreadBytes);
    ChunkBuf<TP>* sBuf = reinterpret_cast<ChunkBuf<TP>*>(after_j + (kFixed ? (blockDim.x >> 5) * kSpreadBytes : 0)) +
                         (threadIdx.x >> 5);
    const int ntiles = t.ntx * t.nty * t.ntz;
    const int T3 = tx * ty * tz;
    const long long N = g.N;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // reciprocals from the host (no FP64 division per thread)
    const TP dt = TP(g.dt), idt = TP(inv_dt);
    const TP dx = TP(g.dx), dy = TP(g.dy), dz = TP(g.dz);
    const TP idx = TP(g.idx), idy = TP(g.idy), idz = TP(g.idz);
    const TP vol = dx * dy * dz;
    const int ey = CT ? 1 : (g.y3 ? 1 : 0), ez = CT ? 1 : (g.z3 ? 1 : 0);
    const int fsy = ey ? fx : 0, fsz = ez ? fx * fy : 0;

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int ti = tile % t.ntx, tj = (tile / t.ntx) % t.nty, tk = tile / (t.ntx * t.nty);
        const int lox = ti * tx, loy = tj * ty, loz = tk * tz;
        for (int e = threadIdx.x; e < F; e += blockDim.x) {
            int a = e % fx, b = (e / fx) % fy, c = e / (fx * fy);
            long long gi = linw(g, lox - hx + a, loy - hy + b, loz - hz + c);
#pragma unroll
            for (int comp = 0; comp < 3; ++comp) {
                sF[comp * F + e] = E[comp * N + gi];
                sF[(3 + comp) * F + e] = B[comp * N + gi];
            }
        }
        if (kFixed) {
            for (long long e = threadIdx.x; e < 3 * JC; e += blockDim.x) { sLo[e] = 0u; sHi[e] = 0; }
        } else {
            for (long long e = threadIdx.x; e < 3 * JC; e += blockDim.x) sJ[e] = TP(0);
        }
        __syncthreads();

        for (int sp = 0; sp < S.ns; ++sp) {
            const PartView<TP> P = S.p[sp];
            const TP q = S.q[sp], m = S.m[sp];
            const TP beta = q * dt / (TP(2) * m);
            const TP fcd = q * S.w[sp] / vol;
            const long long pb = S.off[sp][(long long)tile * T3], pe = S.off[sp][(long long)(tile + 1) * T3];
            // CTA-uniform chunk loop: warp w takes particles cb + 32 w + lane.
            // Each warp's next chunk is copied into its shared buffer while
            // it pushes the current one (the first before the loop).
            if (pb + threadIdx.x < pe) stage_particle(sBuf, P, pb + threadIdx.x, lane);
            cp_async_commit();
            for (long long cb = pb; cb < pe; cb += blockDim.x) {
                const long long n = cb + threadIdx.x;
                TP aB[12];
                TP s1[6] = {TP(0), TP(0), TP(0), TP(0), TP(0), TP(0)};   // F1 and W1 of the old-side segment
                int keyA = -1 - lane, keyB = -1 - lane;   // lanes outside a reduction keep unique keys
                bool push_later = false, deposit_later = false;
                // a lane reads and refills only its own slots, and the wait
                // covers the copies it started itself
                cp_async_wait_all();
                const int cell = n < pe ? sBuf->cell[lane] : -1;
                TP ox = sBuf->a[0][lane], oy = sBuf->a[1][lane], oz = sBuf->a[2][lane];
                TP mom[3] = {sBuf->a[3][lane], sBuf->a[4][lane], sBuf->a[5][lane]};
                if (n + blockDim.x < pe) stage_particle(sBuf, P, n + blockDim.x, lane);
                cp_async_commit();
                // (an escaped particle of a wall box waits with cell -1 for the sort)
                if (n < pe && (!kWall || cell >= 0)) {
                    int i, j, k;
                    decode(g, cell, i, j, k);
                    auto local = [](int c, int lo, int te, int nn) {
                        int l = c - lo;
                        if (l > te) l -= nn;
                        if (l < -1) l += nn;
                        return l;
                    };
                    const int li = local(i, lox, tx, g.nx);
                    const int lj = ey ? local(j, loy, ty, g.ny) : 0;
                    const int lk = ez ? local(k, loz, tz, g.nz) : 0;
                    const bool fast = li >= -1 && li <= tx && lj >= -ey && lj <= ty * ey && lk >= -ez && lk <= tz * ez;
                    push_later = !fast;
                    if (fast) {
                        TP e3[3], b3[3];
                        // upper-neighbour weights: node grids (c, c+1) with weight u;
                        // cell-centred grids (c-1, c) with u + 1/2 below the centre,
                        // (c, c+1) with u - 1/2 above it (correlation.cpp:471-496)
                        const int c0 = (lk + hz) * fsz + (lj + hy) * fsy + (li + hx);
                        const int cxs = ox < TP(0.5) ? -1 : 0;
                        const int cys = (ey && oy < TP(0.5)) ? -fsy : 0;
                        const int czs = (ez && oz < TP(0.5)) ? -fsz : 0;
                        const TP wcx = ox < TP(0.5) ? ox + TP(0.5) : ox - TP(0.5);
                        const TP wcy = ey ? (oy < TP(0.5) ? oy + TP(0.5) : oy - TP(0.5)) : TP(0);
                        const TP wcz = ez ? (oz < TP(0.5) ? oz + TP(0.5) : oz - TP(0.5)) : TP(0);
                        const TP wny = ey ? oy : TP(0), wnz = ez ? oz : TP(0);
                        e3[0] = tri<TP, TF>(sF + 0 * F, c0 + cxs, fsy, fsz, wcx, wny, wnz);
                        e3[1] = tri<TP, TF>(sF + 1 * F, c0 + cys, fsy, fsz, ox, wcy, wnz);
                        e3[2] = tri<TP, TF>(sF + 2 * F, c0 + czs, fsy, fsz, ox, wny, wcz);
                        b3[0] = tri<TP, TF>(sF + 3 * F, c0 + cys + czs, fsy, fsz, ox, wcy, wcz);
                        b3[1] = tri<TP, TF>(sF + 4 * F, c0 + cxs + czs, fsy, fsz, wcx, wny, wcz);
                        b3[2] = tri<TP, TF>(sF + 5 * F, c0 + cxs + cys, fsy, fsz, wcx, wcy, wnz);
                        boris_t<TP>(q, m, dt, beta, e3, b3, mom);
                        TP v[3];
                        velocity_t<TP>(mom, m, v);
                        int ni = i, nj = j, nk = k;
                        int wall_r = 0;
                        if constexpr (kWall) {
                            wall_r = tristan_wall_x<TP>(g, ni, ox, (v[0] * dt) * idx);
                            if (wall_r & 1) { mom[0] = -mom[0]; v[0] = -v[0]; }   // reflectMomentumX
                        } else {
                            advance_axis<TP>(ox, ni, (v[0] * dt) * idx, g.nx);
                        }
                        advance_axis<TP>(oy, nj, (v[1] * dt) * idy, g.ny);
                        advance_axis<TP>(oz, nk, (v[2] * dt) * idz, g.nz);
                        P.px[n] = mom[0]; P.py[n] = mom[1]; P.pz[n] = mom[2];
                        P.ox[n] = ox; P.oy[n] = oy; P.oz[n] = oz;
                        auto shift = [](int nw, int old, int nn) {
                            int d = nw - old;
                            if (d > 1) d -= nn;
                            if (d < -1) d += nn;
                            return d;
                        };
                        // block cell of the new position (a wall box has no x
                        // wrap; a particle reflected from left of the wall may
                        // land far from its old cell and is deposited by the
                        // deferred pass)
                        const int sxw = kWall ? ni - i : shift(ni, i, g.nx);
                        const bool nearx = !kWall || (sxw >= -1 && sxw <= 1);
                        const int bx = li + sxw + hx;
                        const int by = (ey ? lj + shift(nj, j, g.ny) : 0) + hy;
                        const int bz = (ez ? lk + shift(nk, k, g.nz) : 0) + hz;
                        // zigzag split (zig_axis, momentum_collecting.cpp:91-221) in the
                        // new cell's frame: old position P, relay R, relay shift r
                        const TP X = ox * dx, Y = oy * dy, Z = oz * dz;
                        TP PX = X - v[0] * dt;
                        const TP PY = Y - v[1] * dt, PZ = Z - v[2] * dt;
                        if constexpr (kWall) {
                            if (ni == kTristanWallNode && v[0] > TP(0) && PX < TP(0)) PX = -PX;
                        }
                        const int rx = (int)dev_floor(divd<TP>(PX, dx, idx));
                        const int ry = ey ? (int)dev_floor(divd<TP>(PY, dy, idy)) : 0;
                        const int rz = ez ? (int)dev_floor(divd<TP>(PZ, dz, idz)) : 0;
                        const TP RX = rx == 0 ? (X + PX) / TP(2) : TP(rx > 0 ? rx : 0) * dx;
                        const TP RY = ry == 0 ? (Y + PY) / TP(2) : TP(ry > 0 ? ry : 0) * dy;
                        const TP RZ = rz == 0 ? (Z + PZ) / TP(2) : TP(rz > 0 ? rz : 0) * dz;
                        const int ax = bx + rx, ay = by + ry, az = bz + rz;   // block cell of the old-side segment
                        // unsigned compares: (unsigned)x < n is 0 <= x < n
                        const bool inblock = nearx && (unsigned)(rx + 1) <= 2u && (unsigned)(ry + 1) <= 2u &&
                                             (unsigned)(rz + 1) <= 2u && (unsigned)ax < (unsigned)(jx - 1) &&
                                             (unsigned)bx < (unsigned)(jx - 1) && (unsigned)ay < (unsigned)(jy - ey) &&
                                             (unsigned)by < (unsigned)(jy - ey) && (unsigned)az < (unsigned)(jz - ez) &&
                                             (unsigned)bz < (unsigned)(jz - ez);
                        if (inblock) {
                            const TP F1x = divd<TP>(fcd * (RX - PX), dt, idt);
                            const TP F1y = divd<TP>(fcd * (RY - PY), dt, idt);
                            const TP F1z = divd<TP>(fcd * (RZ - PZ), dt, idt);
                            const TP F2x = divd<TP>(fcd * (X - RX), dt, idt);
                            const TP F2y = fcd * v[1] - F1y, F2z = fcd * v[2] - F1z;
                            const TP hxx = TP(0.5) * idx, hyy = TP(0.5) * idy, hzz = TP(0.5) * idz;
                            const TP W1x = divd<TP>(PX + RX, TP(2) * dx, hxx) - TP(rx);
                            const TP W1y = ey ? divd<TP>(PY + RY, TP(2) * dy, hyy) - TP(ry) : TP(0);
                            const TP W1z = ez ? divd<TP>(PZ + RZ, TP(2) * dz, hzz) - TP(rz) : TP(0);
                            const TP W2x = divd<TP>(X + RX, TP(2) * dx, hxx);
                            const TP W2y = ey ? divd<TP>(Y + RY, TP(2) * dy, hyy) : TP(0);
                            const TP W2z = ez ? divd<TP>(Z + RZ, TP(2) * dz, hzz) : TP(0);
                            segment_slots<TP>(F2x, F2y, F2z, W2x, W2y, W2z, aB);
                            s1[0] = F1x; s1[1] = F1y; s1[2] = F1z; s1[3] = W1x; s1[4] = W1y; s1[5] = W1z;
                            keyA = (az * jy + ay) * jx + ax;
                            keyB = (bz * jy + by) * jx + bx;
                        }
                        deposit_later = !inblock;
                        // an escaped particle is marked once its current is
                        // deposited (the deferred pass marks its own)
                        P.cell[n] = ((wall_r & 2) && inblock) ? -1 : (int)lin(g, ni, nj, nk);
                    }
                }
                {
                    const unsigned mp = __ballot_sync(0xffffffffu, push_later);
                    const unsigned md = __ballot_sync(0xffffffffu, deposit_later);
                    if ((mp | md) && lane == 0) {
                        set_defer_bits(S.defer[sp], cb + 32LL * warp, mp);
                        set_defer_bits(S.defer[sp] + S.dwords[sp], cb + 32LL * warp, md);
                    }
                }
                if (keyB < 0) {
#pragma unroll
                    for (int q2 = 0; q2 < 12; ++q2) aB[q2] = TP(0);
                }
                // a particle that stays in its cell (no relay shift) has both
                // segments in that cell: one set of 12 sums carries both, and
                // the old-side pass is left to the particles that crossed (its
                // 12 values are formed only then, from the six kept in s1)
                if (keyA == keyB && keyA >= 0) {
                    TP aA[12];
                    segment_slots<TP>(s1[0], s1[1], s1[2], s1[3], s1[4], s1[5], aA);
#pragma unroll
                    for (int q2 = 0; q2 < 12; ++q2) aB[q2] += aA[q2];
                    keyA = -1 - lane;
                }
                const bool crossed = __any_sync(0xffffffffu, keyA >= 0);
                if constexpr (kFixed) {
                    const bool hb = run_sum<TP>(keyB, aB);
                    add_runs_fx(sLo, sHi, (int)JC, jx, jx * jy, ey, ez, hb, keyB, (const float*)aB, fx_scale, sW);
                } else {
                    if (run_sum<TP>(keyB, aB) && keyB >= 0) add_slots<TP>(sJ, JC, keyB, jx, jx * jy, ey, ez, aB);
                }
                if (crossed) {
                    // lanes without an old-side segment hold unique negative
                    // keys: runs of one lane, whatever their values
                    TP aA[12];
                    segment_slots<TP>(s1[0], s1[1], s1[2], s1[3], s1[4], s1[5], aA);
                    if constexpr (kFixed) {
                        const bool ha = run_sum<TP>(keyA, aA);
                        add_runs_fx(sLo, sHi, (int)JC, jx, jx * jy, ey, ez, ha, keyA, (const float*)aA, fx_scale, sW);
                    } else {
                        if (run_sum<TP>(keyA, aA) && keyA >= 0) add_slots<TP>(sJ, JC, keyA, jx, jx * jy, ey, ez, aA);
                    }
                }
            }
        }
        __syncthreads();
        double* dst = Jpart + (long long)tile * 3 * JC;
        if (kFixed) {
            // the exact block sums as 64-bit integers (k_assemble_j adds
            // them exactly and scales once per cell): integer operations
            // only, nothing on the FP64 pipe
            long long* dsti = reinterpret_cast<long long*>(dst);
            for (long long e = threadIdx.x; e < 3 * JC; e += blockDim.x)
                dsti[e] = (long long)sHi[e] * 4294967296ll + (long long)sLo[e];
        } else {
            for (long long e = threadIdx.x; e < 3 * JC; e += blockDim.x) dst[e] = sJ[e];
        }
        __syncthreads();
    }
}

// The particles k_push_deposit_tile left over, by their mask bits (each
// word read once and cleared for the next step):
//   * push-later (more than one cell outside their tile): the same gather
//     from global memory, Boris push and move, then the zigzag current;
//   * deposit-later (pushed there, segments outside the tile's current
//     block): the zigzag current of the stored new position and velocity.
// The current goes into Jfix with FP64 global atomics; a particle that left a
// wall box is marked (cell -1) once its current is in.
template <typename TP, typename TF>
__global__ void __launch_bounds__(256) k_push_deposit_deferred(GridP g, SpeciesSet<TP> S, const TF* __restrict__ E,
                                                               const TF* __restrict__ B, double* __restrict__ Jfix) {
    const TP dt = TP(g.dt);
    const TP idx = TP(g.idx), idy = TP(g.idy), idz = TP(g.idz);
    const TP vol = TP(g.dx) * TP(g.dy) * TP(g.dz);
    for (int sp = 0; sp < S.ns; ++sp) {
        const PartView<TP> P = S.p[sp];
        const TP q = S.q[sp], m = S.m[sp];
        const TP beta = q * dt / (TP(2) * m);
        const TP fcd = q * S.w[sp] / vol;
        unsigned* mp = S.defer[sp];
        unsigned* md = mp + S.dwords[sp];
        const long long words = (P.n + 31) / 32 + 1;
        for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < words;
             w += (long long)gridDim.x * blockDim.x) {
            unsigned bp = mp[w], bd = md[w];
            if (!(bp | bd)) continue;
            mp[w] = 0u;
            md[w] = 0u;
            while (bp | bd) {
                const bool push = bp != 0u;
                unsigned& bits = push ? bp : bd;
                const long long n = w * 32 + (__ffs(bits) - 1);
                bits &= bits - 1u;
                TP ox = P.ox[n], oy = P.oy[n], oz = P.oz[n];
                TP mom[3] = {P.px[n], P.py[n], P.pz[n]};
                int ni, nj, nk;
                decode(g, P.cell[n], ni, nj, nk);
                TP v[3];
                if (push) {
                    TP e3[3], b3[3];
                    yee_gather<TP, TF>(g, P.cell[n], ox, oy, oz, E, B, e3, b3);
                    boris_t<TP>(q, m, dt, beta, e3, b3, mom);
                    velocity_t<TP>(mom, m, v);
                    if (g.wall) {
                        if (tristan_wall_x<TP>(g, ni, ox, (v[0] * dt) * idx) & 1) {   // reflectMomentumX
                            mom[0] = -mom[0];
                            v[0] = -v[0];
                        }
                    } else {
                        advance_axis<TP>(ox, ni, (v[0] * dt) * idx, g.nx);
                    }
                    advance_axis<TP>(oy, nj, (v[1] * dt) * idy, g.ny);
                    advance_axis<TP>(oz, nk, (v[2] * dt) * idz, g.nz);
                    P.px[n] = mom[0]; P.py[n] = mom[1]; P.pz[n] = mom[2];
                    P.ox[n] = ox; P.oy[n] = oy; P.oz[n] = oz;
                } else {
                    velocity_t<TP>(mom, m, v);
                }
                deposit_global<TP>(g, fcd, ox, oy, oz, v, ni, nj, nk, Jfix);
                P.cell[n] = (g.wall && tristan_escaped<TP>(g, ni, ox)) ? -1 : (int)lin(g, ni, nj, nk);
            }
        }
    }
}

// J[c] = Jfix[c] + sum of every tile partial that covers cell c, tiles and
// periodic images visited in a fixed order (deterministic).  FP32 particles:
// the partials are 64-bit fixed-point integers, summed exactly and scaled by
// inv_scale (a power of two) once; FP64 particles: FP64 partials.
template <typename TP>
__global__ void __launch_bounds__(256) k_assemble_j(GridP g, TileGeom t, TileShape s, const double* __restrict__ Jpart,
                                                    const double* __restrict__ Jfix, double* __restrict__ J,
                                                    double inv_scale) {
    constexpr bool kFixed = sizeof(TP) == sizeof(float);
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
        long long iacc[3] = {0, 0, 0};
        for (int a = 0; a < cnt[0]; ++a)
            for (int b = 0; b < cnt[1]; ++b)
                for (int d = 0; d < cnt[2]; ++d) {
                    long long tile = ((long long)cand_t[2][d] * t.nty + cand_t[1][b]) * t.ntx + cand_t[0][a];
                    long long e = ((long long)cand_l[2][d] * s.jy + cand_l[1][b]) * s.jx + cand_l[0][a];
                    const double* src = Jpart + tile * 3 * JC;
                    if constexpr (kFixed) {
                        const long long* srci = reinterpret_cast<const long long*>(src);
                        iacc[0] += srci[e];
                        iacc[1] += srci[JC + e];
                        iacc[2] += srci[2 * JC + e];
                    } else {
                        acc[0] += src[e];
                        acc[1] += src[JC + e];
                        acc[2] += src[2 * JC + e];
                    }
                }
        if constexpr (kFixed) {
#pragma unroll
            for (int q = 0; q < 3; ++q) acc[q] += (double)iacc[q] * inv_scale;
        }
        J[c] = acc[0]; J[g.N + c] = acc[1]; J[2 * g.N + c] = acc[2];
    }
}

}  // namespace pic
