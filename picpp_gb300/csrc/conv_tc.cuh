// conv_tc.cuh -- 3x3x3 convolution of the learned preconditioner on the
// 5th-generation tensor cores (tcgen05.mma, BF16 operands from shared
// memory, FP32 accumulator in tensor memory).
//
// One CTA computes a 1 x 16 x 8 (d, h, w) output brick: M = 128 voxels,
// N = COUT, K = 27 taps x CIN.  The input brick with its one-voxel halo
// (3 x 18 x 10 voxels) sits in shared memory in the no-swizzle K-major
// "core matrix" layout of the tensor cores: [CIN/8][voxel][8 channels], so
// 8 voxels adjacent in w with 8 channels are one contiguous 128-byte core
// matrix.  A tap (kd, kh, kw) shifts the brick by whole voxels, which only
// moves the start address of the A descriptor: the 16 rows of 8 voxels of
// the output brick are core matrices 10 voxels (one brick row) apart.  No
// im2col copy exists.  The weights of a tap are [CIN/8][COUT][8] core
// matrices (B, K-major).  One thread issues the MMAs (K = 16 each) and
// commits them to an mbarrier; the epilogue reads the accumulator rows
// back with tcgen05.ld (warp w reads TMEM lanes 32 (w % 4) .. + 31), adds
// the bias, applies ReLU and writes BF16 and/or FP32 NDHWC outputs.
// Every wait is bounded; a wait that runs out sets *err and the CTA still
// releases its tensor memory.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace pic {
namespace nn {

constexpr int kTcH = 16, kTcW = 8;                        // output brick (d extent 1)
constexpr int kTcBD = 3, kTcBH = kTcH + 2, kTcBW = kTcW + 2;
constexpr int kTcBV = kTcBD * kTcBH * kTcBW;              // 540 brick voxels
constexpr int kTcThreads = 256;
constexpr unsigned kTcWaitLimit = 1u << 22;               // mbarrier polls before giving up

// All 27 taps of weights staged at once when they fit next to the brick;
// otherwise one kd plane (9 taps) at a time.
__host__ __device__ constexpr bool tc_all_taps(int cin, int cout) {
    return (27 * (size_t)cin * cout + (size_t)cin * kTcBV) * 2 <= 64 * 1024;
}
__host__ __device__ constexpr size_t tc_conv_smem_bytes(int cin, int cout) {
    return ((size_t)cin * kTcBV + (tc_all_taps(cin, cout) ? 27 : 9) * (size_t)cin * cout) * 2;
}
__host__ __device__ constexpr int tc_tmem_cols(int cout) { return cout <= 32 ? 32 : (cout <= 64 ? 64 : 128); }

// Shared-memory matrix descriptor, no swizzle: start address, leading
// (K-direction) and stride (M/N-direction) byte offsets between core
// matrices, descriptor version 1 (bit 46).
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1),
// BF16 A and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17,
// M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int accum) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity, unsigned limit = kTcWaitLimit) {
    for (unsigned it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred P1;\n mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
            " selp.b32 %0, 1, 0, P1;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// The same wait with a poll count that means polls: test_wait returns at
// once, where one try_wait may itself block for a hardware-chosen time.
__device__ __forceinline__ bool tc_poll(uint32_t mbar, uint32_t parity, unsigned polls) {
    for (unsigned it = 0; it < polls; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred P1;\n mbarrier.test_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
            " selp.b32 %0, 1, 0, P1;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 8 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld8(uint32_t taddr, float v[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// 16-byte asynchronous copy global -> shared through L1 (neighbouring bricks
// share their halos, every CTA the weights); src_bytes = 0 writes zeros
// (the halo outside the box).  All of a thread's copies are in flight at
// once instead of one load-store round trip per item.
__device__ __forceinline__ void tc_cp16(void* dst, const void* src, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void tc_cp_wait_all() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// y[v][co] = bias[co] + sum_tap sum_ci x[v + off(tap)][ci] * Wk[tap][co][ci]
// (zero outside the box), then optional ReLU; BF16 (y16) and/or FP32 (y32).
// Dims {N, D, H, W}; NDHWC activations with CIN / COUT channels.
template <int CIN, int COUT>
__global__ void __launch_bounds__(kTcThreads) k_conv3_tc(const __nv_bfloat16* __restrict__ x,
                                                         const __nv_bfloat16* __restrict__ Wk,
                                                         const float* __restrict__ bias,
                                                         __nv_bfloat16* __restrict__ y16, float* __restrict__ y32,
                                                         int dN, int dD, int dH, int dW, int relu,
                                                         int* __restrict__ err, unsigned wait_limit) {
    static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT <= 128, "channel counts");
    constexpr int C8 = CIN / 8;
    constexpr bool kAll = tc_all_taps(CIN, COUT);
    constexpr int kStages = kAll ? 1 : 3;
    constexpr int kTapsPerStage = kAll ? 27 : 9;
    constexpr int kCols = tc_tmem_cols(COUT);
    constexpr uint32_t kIdesc = tc_idesc(128, COUT);
    extern __shared__ __align__(128) unsigned char tc_smem[];
    __shared__ __align__(8) unsigned long long s_mbar;
    __shared__ uint32_t s_tmem;
    __nv_bfloat16* sA = reinterpret_cast<__nv_bfloat16*>(tc_smem);   // [C8][kTcBV][8]
    __nv_bfloat16* sW = sA + (size_t)CIN * kTcBV;                      // [taps][C8][COUT][8]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w0 = blockIdx.x * kTcW, h0 = blockIdx.y * kTcH;
    const int n = blockIdx.z / dD, d0 = blockIdx.z % dD;
    const uint32_t mbar = (uint32_t)__cvta_generic_to_shared(&s_mbar);

    if (warp == 0) {
        const uint32_t slot = (uint32_t)__cvta_generic_to_shared(&s_tmem);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(slot), "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (threadIdx.x == 32) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // input brick: voxels (d0 - 1 .. d0 + 1, h0 - 1 .. h0 + 16, w0 - 1 .. w0 + 8), 16 bytes per copy
    for (int e = threadIdx.x; e < kTcBV * C8; e += kTcThreads) {
        const int bv = e / C8, c8 = e - bv * C8;
        const int bw = bv % kTcBW, bh = (bv / kTcBW) % kTcBH, bd = bv / (kTcBW * kTcBH);
        const int d = d0 - 1 + bd, h = h0 - 1 + bh, w = w0 - 1 + bw;
        const bool in = d >= 0 && d < dD && h >= 0 && h < dH && w >= 0 && w < dW;
        const __nv_bfloat16* src = in ? x + ((((long long)n * dD + d) * dH + h) * dW + w) * CIN + c8 * 8 : x;
        tc_cp16(sA + ((size_t)c8 * kTcBV + bv) * 8, src, in ? 16 : 0);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t aBase = (uint32_t)__cvta_generic_to_shared(sA);
    const uint32_t wBase = (uint32_t)__cvta_generic_to_shared(sW);
    bool ok = true;

    for (int st = 0; st < kStages; ++st) {
        // weights of this stage's taps: Wk[tap][co][ci] -> sW[tap'][ci/8][co][8]
        const __nv_bfloat16* wsrc = Wk + (size_t)st * kTapsPerStage * COUT * CIN;
        for (int e = threadIdx.x; e < kTapsPerStage * COUT * C8; e += kTcThreads) {
            const int row = e / C8, c8 = e - row * C8;   // row = tap' * COUT + co
            const int tp = row / COUT, co = row - tp * COUT;
            tc_cp16(sW + (((size_t)tp * C8 + c8) * COUT + co) * 8, wsrc + (size_t)row * CIN + c8 * 8, 16);
        }
        tc_cp_wait_all();   // this stage's weights (and, at stage 0, the brick) in shared memory
        // generic-proxy writes -> visible to the tensor cores
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (threadIdx.x == 0 && ok) {
            // descriptor start fields count 16-byte units (one voxel of the
            // A layout, one 8-channel row of B): base descriptors plus
            // constants per tap
            const uint64_t aD = tc_desc(aBase, kTcBV * 16, kTcBW * 16);
            const uint64_t bD = tc_desc(wBase, COUT * 16, 128);
#pragma unroll
            for (int tp = 0; tp < kTapsPerStage; ++tp) {
                const int kd = kAll ? tp / 9 : st, kh = (tp / 3) % 3, kw = tp % 3;
                const uint64_t aT = aD + (uint64_t)((kd * kTcBH + kh) * kTcBW + kw);
                const uint64_t bT = bD + (uint64_t)(tp * C8 * COUT);
#pragma unroll
                for (int kc = 0; kc < CIN / 16; ++kc)
                    tc_mma(tmem, aT + (uint64_t)(2 * kc * kTcBV), bT + (uint64_t)(2 * kc * COUT), kIdesc,
                           ((st * kTapsPerStage + tp) | kc) != 0);
            }
            tc_commit(mbar);
        }
        __syncwarp();
        // every thread waits: the next stage overwrites the weights, the
        // epilogue reads TMEM; the outcome is made CTA-uniform.  A nonzero
        // wait_limit bounds this completion wait to that many non-blocking
        // polls (0: kTcWaitLimit blocking polls); the wait before the tensor
        // memory is released below always takes the full bound
        const bool done = wait_limit ? tc_poll(mbar, (uint32_t)(st & 1), wait_limit)
                                     : tc_wait(mbar, (uint32_t)(st & 1));
        ok = __syncthreads_and(done) != 0;
        tc_fence_after();
        if (!ok) {
            if (threadIdx.x == 0 && err) atomicExch(err, 1);
            // give the MMAs in flight another bounded wait before the memory is released
            tc_wait(mbar, (uint32_t)(st & 1));
            break;
        }
    }

    if (ok) {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (accumulator rows), half (w / 4) of the columns
        const int q = warp & 3, half = warp >> 2;
        const int m = 32 * q + lane;
        const int h = h0 + m / kTcW, w = w0 + m % kTcW;
        const bool inside = h < dH && w < dW;
        const long long o = ((((long long)n * dD + d0) * dH + h) * dW + w) * COUT;
        constexpr int kHalfCols = COUT / 2;
#pragma unroll
        for (int c0 = half * kHalfCols; c0 < (half + 1) * kHalfCols; c0 += 8) {
            float v[8];
            tc_ld8(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, v);
            if (!inside) continue;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                if (bias) v[i] += bias[c0 + i];
                if (relu) v[i] = fmaxf(v[i], 0.f);
            }
            if (y16) {
                __align__(16) __nv_bfloat162 p[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) p[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
                *reinterpret_cast<uint4*>(y16 + o + c0) = *reinterpret_cast<const uint4*>(p);
            }
            if (y32) {
                *reinterpret_cast<float4*>(y32 + o + c0) = make_float4(v[0], v[1], v[2], v[3]);
                *reinterpret_cast<float4*>(y32 + o + c0 + 4) = make_float4(v[4], v[5], v[6], v[7]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kCols) : "memory");
    }
}

}  // namespace nn
}  // namespace pic
