// sort.cuh -- stable, deterministic counting sort of particles by cell.
//
// The reference keeps particles in an unordered std::vector<Particle*>; the
// GPU keeps each species in SoA arrays ordered by a tile-major cell key so
// that a tile's particles are contiguous.  The sort is bit-exact with the
// oracle's stable counting sort:
//   1. key per particle, histogram (integer atomics per run of equal keys
//      in a warp: exact counts)
//   2. exclusive scan of the counts (3-phase block scan)
//   3. scatter of source indices with one atomic cursor per key and run
//      (arbitrary order inside a key), then
//   4. per-key segment sort of the source indices by rank counting, which
//      restores input order inside every key: stable and run-independent
//   5. gather of the payload arrays through the permutation.
#pragma once
#include <climits>
#include "common.cuh"
#include "types.cuh"

namespace pic {

__device__ __forceinline__ int sort_key(const GridP& g, const TileGeom& t, int cell) {
    int i, j, k;
    decode(g, cell, i, j, k);
    int ti, tj, tk;
    if (t.lx >= 0) {   // power-of-two tiles (the default): shifts, not divisions
        ti = i >> t.lx; tj = j >> t.ly; tk = k >> t.lz;
    } else {
        ti = i / t.tx; tj = j / t.ty; tk = k / t.tz;
    }
    int li = i - ti * t.tx, lj = j - tj * t.ty, lk = k - tk * t.tz;
    int tile = (tk * t.nty + tj) * t.ntx + ti;
    int local = (lk * t.ty + lj) * t.tx + li;
    return tile * (t.tx * t.ty * t.tz) + local;
}

// Runs of equal keys within a warp: the head lane of each run and the run's
// length (consecutive particles mostly share a key: the input is the
// previous sort order; a key that recurs later in the warp starts another
// run).
__device__ __forceinline__ bool key_run(int kk, int lane, int& len) {
    const int prev = __shfl_up_sync(0xffffffffu, kk, 1);
    const bool head = lane == 0 || kk != prev;
    const unsigned H = __ballot_sync(0xffffffffu, head);
    const unsigned after = H & ~((2u << lane) - 1u);   // heads after this lane
    len = (after ? __ffs(after) - 1 : 32) - lane;
    return head;
}

// Sort key of every particle and the per-key counts, one atomic per run of
// equal keys in a warp.
__global__ void k_keys_hist(GridP g, TileGeom t, const int* __restrict__ cell, long long n, int* __restrict__ key,
                            int* __restrict__ counts) {
    const int lane = threadIdx.x & 31;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long base = ((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5) * 32; base < n; base += nw * 32) {
        const long long a = base + lane;
        const int ca = a < n ? cell[a] : -1;   // escaped particles (cell -1) get no key and drop out
        const int kk = ca >= 0 ? sort_key(g, t, ca) : -1;
        if (a < n) key[a] = kk;
        int len;
        if (key_run(kk, lane, len) && kk >= 0) atomicAdd(&counts[kk], len);
    }
}

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;   // per thread -> 2048 per block

__device__ __forceinline__ int block_excl_scan(int v, int* sh, int& total) {
    // warp inclusive scan
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int s = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sh[lane] = s;   // inclusive warp totals
    }
    __syncthreads();
    int warp_off = wid > 0 ? sh[wid - 1] : 0;
    total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_off + x - v;
}

// in-place exclusive scan, phase 1: per-block scan, block totals out.
__global__ void __launch_bounds__(kScanThreads) k_scan_blocks(int* __restrict__ a, long long n, int* __restrict__ block_sums) {
    __shared__ int sh[32];
    long long base = (long long)blockIdx.x * kScanThreads * kScanItems + (long long)threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) {
        v[q] = (base + q < n) ? a[base + q] : 0;
        s += v[q];
    }
    int total;
    int off = block_excl_scan(s, sh, total);
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) {
        if (base + q < n) a[base + q] = off;
        off += v[q];
    }
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// phase 2: exclusive scan of the block totals by one block (any count).
__global__ void __launch_bounds__(kScanThreads) k_scan_top(int* __restrict__ s, int nb, int* __restrict__ grand_total) {
    __shared__ int sh[32];
    int carry = 0;
    for (int base = 0; base < nb; base += kScanThreads) {
        int idx = base + threadIdx.x;
        int v = idx < nb ? s[idx] : 0;
        int total;
        int off = block_excl_scan(v, sh, total);
        if (idx < nb) s[idx] = carry + off;
        carry += total;
    }
    if (threadIdx.x == 0 && grand_total) *grand_total = carry;
}

// phase 3: add block offsets.
__global__ void __launch_bounds__(kScanThreads) k_scan_add(int* __restrict__ a, long long n, const int* __restrict__ block_sums) {
    long long base = (long long)blockIdx.x * kScanThreads * kScanItems;
    int add = block_sums[blockIdx.x];
    for (int q = threadIdx.x; q < kScanThreads * kScanItems; q += kScanThreads)
        if (base + q < n) a[base + q] += add;
}

// Source index a to tmp[cursor[key[a]]++], one atomic per run of equal keys
// in a warp; the order inside a key is restored by the segment sort.
__global__ void k_scatter_atomic(const int* __restrict__ key, long long n, int* __restrict__ cursor, int* __restrict__ tmp) {
    const int lane = threadIdx.x & 31;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long base = ((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5) * 32; base < n; base += nw * 32) {
        const long long a = base + lane;
        const int kk = a < n ? key[a] : -1;
        int len;
        const bool head = key_run(kk, lane, len);
        int pos = 0;
        if (head && kk >= 0) pos = atomicAdd(&cursor[kk], len);
        // each lane takes its run head's position plus its place in the run
        const unsigned H = __ballot_sync(0xffffffffu, head);
        const int hl = 31 - __clz(H & ((2u << lane) - 1u));   // this lane's head
        pos = __shfl_sync(0xffffffffu, pos, hl);
        if (kk >= 0) tmp[pos + (lane - hl)] = (int)a;
    }
}

// Ascending sort of one segment of up to 32 R distinct source indices held
// by a warp, element i = 32 r + lane in v[r] (padding INT_MAX): bitonic
// network, exchanges across lanes by shuffles and across registers in place.
template <int R>
__device__ __forceinline__ void warp_bitonic(int v[R], int lane) {
#pragma unroll
    for (int k = 2; k <= 32 * R; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                const int jr = j >> 5;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if (r & jr) continue;
                    const bool up = (((32 * r + lane) & k) == 0);
                    const int lo = min(v[r], v[r | jr]), hi = max(v[r], v[r | jr]);
                    v[r] = up ? lo : hi;
                    v[r | jr] = up ? hi : lo;
                }
            } else {
                const bool lower = (lane & j) == 0;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int y = __shfl_xor_sync(0xffffffffu, v[r], j);
                    const bool up = (((32 * r + lane) & k) == 0);
                    v[r] = (lower == up) ? min(v[r], y) : max(v[r], y);
                }
            }
        }
    }
}

// One segment [b, b + len) of tmp, 32 R >= len, sorted into perm by a warp:
// copied when already ascending (the scatter keeps each warp's particles in
// order, so a segment filled by one warp, or by warps in index order, is),
// else sorted in registers.
template <int R>
__device__ __forceinline__ void warp_sort_segment(const int* __restrict__ tmp, int* __restrict__ perm, int b, int len,
                                                  int lane) {
    int v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = 32 * r + lane < len ? tmp[b + 32 * r + lane] : INT_MAX;
    bool sorted = true;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int nx = __shfl_down_sync(0xffffffffu, v[r], 1);
        const int first_next = r + 1 < R ? __shfl_sync(0xffffffffu, v[r + 1 < R ? r + 1 : r], 0) : INT_MAX;
        const int next = lane < 31 ? nx : first_next;
        if (32 * r + lane + 1 < len && v[r] > next) sorted = false;
    }
    if (!__all_sync(0xffffffffu, sorted)) warp_bitonic<R>(v, lane);
#pragma unroll
    for (int r = 0; r < R; ++r)
        if (32 * r + lane < len) perm[b + 32 * r + lane] = v[r];
}

// Stable order of each key segment [off[k], off[k+1]) of tmp into perm
// (ascending source index).  Segments up to kWarpSeg elements use one warp;
// longer ones are left to k_segsort_block.
constexpr int kWarpSeg = 256;
__global__ void k_segsort_warp(const int* __restrict__ off, int nkeys, const int* __restrict__ tmp, int* __restrict__ perm,
                               int* __restrict__ long_count, int* __restrict__ long_list) {
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long kk = warp; kk < nkeys; kk += nwarps) {
        int b = off[kk], e = off[kk + 1];
        int len = e - b;
        if (len <= 0) continue;
        if (len == 1) { if (lane == 0) perm[b] = tmp[b]; continue; }
        if (len > kWarpSeg) {
            if (lane == 0) { int slot = atomicAdd(long_count, 1); long_list[slot] = (int)kk; }
            continue;
        }
        if (len <= 32) warp_sort_segment<1>(tmp, perm, b, len, lane);
        else if (len <= 64) warp_sort_segment<2>(tmp, perm, b, len, lane);
        else if (len <= 128) warp_sort_segment<4>(tmp, perm, b, len, lane);
        else warp_sort_segment<8>(tmp, perm, b, len, lane);
    }
}

__global__ void k_segsort_block(const int* __restrict__ off, const int* __restrict__ long_list, const int* __restrict__ long_count,
                                const int* __restrict__ tmp, int* __restrict__ perm) {
    const int cnt = *long_count;
    for (int s = blockIdx.x; s < cnt; s += gridDim.x) {
        int kk = long_list[s];
        int b = off[kk], e = off[kk + 1];
        int len = e - b;
        for (int a = threadIdx.x; a < len; a += blockDim.x) {
            int x = tmp[b + a];
            int r = 0;
            for (int c = 0; c < len; ++c) r += tmp[b + c] < x;
            perm[b + r] = x;
        }
    }
}

}  // namespace pic
