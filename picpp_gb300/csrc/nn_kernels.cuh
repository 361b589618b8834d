// nn_kernels.cuh -- kernels of the learned preconditioner's network: 3x3x3
// convolutions as implicit GEMMs on the BF16 tensor cores (FP32
// accumulation), pooling / upsampling / skip concatenation, their
// backward passes, weight gradients, the loss and Adam.
//
// Activations are NDHWC BF16 with channel counts that are multiples of 16;
// a voxel's channels are one contiguous 16-byte-aligned run.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace pic {
namespace nn {

using bf16 = __nv_bfloat16;

struct Dims {
    int N, D, H, W;
    __host__ __device__ long long vox() const { return (long long)N * D * H * W; }
};

// Output brick of one conv CTA: 2 x 8 x 8 voxels, 16 per warp.
constexpr int kBD = 2, kBH = 8, kBW = 8;
constexpr int kHD = kBD + 2, kHH = kBH + 2, kHW = kBW + 2;
constexpr int kHalo = kHD * kHH * kHW;
constexpr int kConvThreads = 256;

// Shared memory of one conv CTA: the input brick with halo and one plane
// (9 taps) of weights, both with row stride CIN + 8 BF16.
__host__ __device__ constexpr size_t conv_smem_bytes(int cin, int cout) {
    return ((size_t)kHalo + 9 * (size_t)cout) * (cin + 8) * 2;
}

__device__ __forceinline__ void ldsm_x4(unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3, const void* p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a));
}

__device__ __forceinline__ void ldsm_x2(unsigned& r0, unsigned& r1, const void* p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}

__device__ __forceinline__ void mma_bf16_16816(float c[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                               unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// y[v][co] = bias[co] + sum_tap sum_ci x[v + off(tap)][ci] * Wk[tap][co][ci]
// (zero outside the box), then optional ReLU; written as BF16 (y16) and/or
// FP32 (y32).  GEMM per CTA: M = 128 voxels (8 warps x m16), N = COUT, K =
// 27 taps x CIN.  The input brick plus a one-voxel halo and, plane by plane
// (kd = 0, 1, 2), the nine taps' weights are staged in shared memory with
// row stride CIN + 8 BF16 (conflict-free ldmatrix for A and B fragments).
template <int CIN, int COUT>
__global__ void __launch_bounds__(kConvThreads) k_conv3(const bf16* __restrict__ x, const bf16* __restrict__ Wk,
                                                        const float* __restrict__ bias, bf16* __restrict__ y16,
                                                        float* __restrict__ y32, Dims dm, int relu) {
    static_assert(CIN % 16 == 0 && COUT % 16 == 0, "channel counts");
    constexpr int SST = CIN + 8;
    constexpr int NT = COUT / 8;
    constexpr int C8 = CIN / 8;
    extern __shared__ __align__(16) unsigned char conv_smem[];
    bf16* sx = reinterpret_cast<bf16*>(conv_smem);   // [kHalo][SST]
    bf16* sw = sx + kHalo * SST;                     // [9][COUT][SST]
    const int nbd = (dm.D + kBD - 1) / kBD;
    const int w0 = blockIdx.x * kBW, h0 = blockIdx.y * kBH;
    const int n = blockIdx.z / nbd, d0 = (blockIdx.z % nbd) * kBD;
    // stage the halo brick, 8 channels (16 bytes) per access
    for (int e = threadIdx.x; e < kHalo * C8; e += kConvThreads) {
        const int hv = e / C8, c8 = e - hv * C8;
        const int hw = hv % kHW, hh = (hv / kHW) % kHH, hd = hv / (kHW * kHH);
        const int d = d0 - 1 + hd, h = h0 - 1 + hh, w = w0 - 1 + hw;
        uint4 val = make_uint4(0, 0, 0, 0);
        if (d >= 0 && d < dm.D && h >= 0 && h < dm.H && w >= 0 && w < dm.W)
            val = *reinterpret_cast<const uint4*>(x + ((((long long)n * dm.D + d) * dm.H + h) * dm.W + w) * CIN + c8 * 8);
        *reinterpret_cast<uint4*>(sx + hv * SST + c8 * 8) = val;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    // ldmatrix row of this lane: voxel r = lane % 16 of the warp's 16
    const int r = lane & 15;
    const int v = warp * 16 + r;
    const int vd = v / (kBH * kBW), vh = (v / kBW) % kBH, vw = v % kBW;
    const int koff = (lane >> 4) * 8;
    // B fragments: lanes 0-7 rows co of k half 0, lanes 8-15 k half 1,
    // lanes 16-31 the same for the next n-tile
    const int brow = (lane & 7) + ((lane >> 4) << 3);
    const int bk = ((lane >> 3) & 1) * 8;
    float acc[NT][4];
#pragma unroll
    for (int i = 0; i < NT; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll 1
    for (int kd = 0; kd < 3; ++kd) {
        __syncthreads();   // previous plane's weights consumed (and, for kd = 0, the halo staged)
        const bf16* wsrc = Wk + (size_t)kd * 9 * COUT * CIN;
        for (int e = threadIdx.x; e < 9 * COUT * C8; e += kConvThreads) {
            const int row = e / C8, c8 = e - row * C8;   // row = tap_in_plane * COUT + co
            *reinterpret_cast<uint4*>(sw + row * SST + c8 * 8) =
                *reinterpret_cast<const uint4*>(wsrc + (size_t)row * CIN + c8 * 8);
        }
        __syncthreads();
#pragma unroll 1
        for (int tp = 0; tp < 9; ++tp) {
            const int kh = tp / 3, kw = tp % 3;
            const bf16* arow = sx + (((vd + kd) * kHH + (vh + kh)) * kHW + (vw + kw)) * SST + koff;
            const bf16* wt = sw + (size_t)tp * COUT * SST;
#pragma unroll
            for (int k0 = 0; k0 < CIN; k0 += 16) {
                unsigned a0, a1, a2, a3;
                ldsm_x4(a0, a1, a2, a3, arow + k0);
#pragma unroll
                for (int nt = 0; nt < NT; nt += 2) {
                    unsigned b0, b1, b2, b3;
                    ldsm_x4(b0, b1, b2, b3, wt + (nt * 8 + brow) * SST + k0 + bk);
                    mma_bf16_16816(acc[nt], a0, a1, a2, a3, b0, b1);
                    mma_bf16_16816(acc[nt + 1], a0, a1, a2, a3, b2, b3);
                }
            }
        }
    }
    // epilogue: rows g and g + 8 of the warp's 16 voxels
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const int vv = warp * 16 + g + half * 8;
        const int d = d0 + vv / (kBH * kBW), h = h0 + (vv / kBW) % kBH, w = w0 + vv % kBW;
        if (d >= dm.D || h >= dm.H || w >= dm.W) continue;
        const long long o = ((((long long)n * dm.D + d) * dm.H + h) * dm.W + w) * COUT;
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const int co = nt * 8 + 2 * t;
            float y0 = acc[nt][2 * half], y1 = acc[nt][2 * half + 1];
            if (bias) { y0 += bias[co]; y1 += bias[co + 1]; }
            if (relu) { y0 = fmaxf(y0, 0.f); y1 = fmaxf(y1, 0.f); }
            if (y16) *reinterpret_cast<__nv_bfloat162*>(y16 + o + co) = __floats2bfloat162_rn(y0, y1);
            if (y32) *reinterpret_cast<float2*>(y32 + o + co) = make_float2(y0, y1);
        }
    }
}

// dW[tap][co][ci] += sum_v x[v + off(tap)][ci] * gy[v][co], and (blocks of
// tap 0) db[co] += sum_v gy[v][co]; FP32 partial sums over a chunk of 128
// voxels per CTA, added with global atomics.
constexpr int kWgVox = 128;
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_wgrad(const bf16* __restrict__ x, const bf16* __restrict__ gy, Dims dm,
                                               float* __restrict__ dW, float* __restrict__ db) {
    constexpr int PER = CIN * COUT / 256;
    extern __shared__ __align__(16) unsigned char wg_smem[];
    float* sx = reinterpret_cast<float*>(wg_smem);   // [kWgVox][CIN]
    float* sg = sx + kWgVox * CIN;                   // [kWgVox][COUT]
    const int tap = blockIdx.y;
    const int kd = tap / 9 - 1, kh = (tap / 3) % 3 - 1, kw = tap % 3 - 1;
    const long long V = dm.vox();
    const long long v0 = (long long)blockIdx.x * kWgVox;
    for (int e = threadIdx.x; e < kWgVox * CIN; e += 256) {
        const int vi = e / CIN, ci = e % CIN;
        const long long v = v0 + vi;
        float val = 0.f;
        if (v < V) {
            const int w = (int)(v % dm.W), h = (int)((v / dm.W) % dm.H), d = (int)((v / ((long long)dm.W * dm.H)) % dm.D);
            const long long nn = v / ((long long)dm.W * dm.H * dm.D);
            const int dd = d + kd, hh = h + kh, ww = w + kw;
            if (dd >= 0 && dd < dm.D && hh >= 0 && hh < dm.H && ww >= 0 && ww < dm.W)
                val = __bfloat162float(x[(((nn * dm.D + dd) * dm.H + hh) * dm.W + ww) * CIN + ci]);
        }
        sx[e] = val;
    }
    for (int e = threadIdx.x; e < kWgVox * COUT; e += 256) {
        const long long v = v0 + e / COUT;
        sg[e] = v < V ? __bfloat162float(gy[v * COUT + e % COUT]) : 0.f;
    }
    __syncthreads();
    float acc[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) acc[j] = 0.f;
    for (int vi = 0; vi < kWgVox; ++vi) {
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const int el = threadIdx.x + 256 * j;
            const int co = el / CIN, ci = el % CIN;
            acc[j] += sx[vi * CIN + ci] * sg[vi * COUT + co];
        }
    }
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const int el = threadIdx.x + 256 * j;
        atomicAdd(&dW[(size_t)tap * COUT * CIN + el], acc[j]);
    }
    if (tap == 0 && threadIdx.x < COUT) {
        float s = 0.f;
        for (int vi = 0; vi < kWgVox; ++vi) s += sg[vi * COUT + threadIdx.x];
        atomicAdd(&db[threadIdx.x], s);
    }
}

// 2x2x2 average pooling (NDHWC, C channels), dims of the input.
__global__ void k_pool(const bf16* __restrict__ x, bf16* __restrict__ y, Dims di, int C) {
    const int D2 = di.D / 2, H2 = di.H / 2, W2 = di.W / 2;
    const long long tot = (long long)di.N * D2 * H2 * W2 * C;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        long long v = e / C;
        const int w = (int)(v % W2), h = (int)((v / W2) % H2), d = (int)((v / ((long long)W2 * H2)) % D2);
        const long long n = v / ((long long)W2 * H2 * D2);
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int dd = 2 * d + (q >> 2), hh = 2 * h + ((q >> 1) & 1), ww = 2 * w + (q & 1);
            s += __bfloat162float(x[(((n * di.D + dd) * di.H + hh) * di.W + ww) * C + c]);
        }
        y[e] = __float2bfloat16(s * 0.125f);
    }
}

// y[v] = concat(lo[v / 2] (C1 channels, nearest upsampling), skip[v] (C2)),
// dims of the fine level.
__global__ void k_up_concat(const bf16* __restrict__ lo, const bf16* __restrict__ skip, bf16* __restrict__ y, Dims df,
                            int C1, int C2) {
    const int C = C1 + C2;
    const long long tot = df.vox() * C;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const long long v = e / C;
        if (c >= C1) { y[e] = skip[v * C2 + (c - C1)]; continue; }
        const int w = (int)(v % df.W), h = (int)((v / df.W) % df.H), d = (int)((v / ((long long)df.W * df.H)) % df.D);
        const long long n = v / ((long long)df.W * df.H * df.D);
        const long long vl = ((n * (df.D / 2) + d / 2) * (df.H / 2) + h / 2) * (df.W / 2) + w / 2;
        y[e] = lo[vl * C1 + c];
    }
}

// Backward of k_up_concat: glo[vl] = sum of the 8 children's first C1
// channels; gskip[v] = the last C2 channels (FP32; dims of the fine level).
__global__ void k_up_concat_bwd(const float* __restrict__ gy, float* __restrict__ glo, float* __restrict__ gskip,
                                Dims df, int C1, int C2) {
    const int C = C1 + C2;
    const long long tot_skip = df.vox() * C2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot_skip;
         e += (long long)gridDim.x * blockDim.x) {
        const long long v = e / C2;
        gskip[e] = gy[v * C + C1 + e % C2];
    }
    const int D2 = df.D / 2, H2 = df.H / 2, W2 = df.W / 2;
    const long long tot_lo = (long long)df.N * D2 * H2 * W2 * C1;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot_lo; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C1);
        const long long v = e / C1;
        const int w = (int)(v % W2), h = (int)((v / W2) % H2), d = (int)((v / ((long long)W2 * H2)) % D2);
        const long long n = v / ((long long)W2 * H2 * D2);
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int dd = 2 * d + (q >> 2), hh = 2 * h + ((q >> 1) & 1), ww = 2 * w + (q & 1);
            s += gy[(((n * df.D + dd) * df.H + hh) * df.W + ww) * C + c];
        }
        glo[e] = s;
    }
}

// gfine[v] += gcoarse[v / 2] / 8 (backward of the average pooling; dims of
// the fine level).
__global__ void k_pool_bwd_add(const float* __restrict__ gc, float* __restrict__ gf, Dims df, int C) {
    const long long tot = df.vox() * C;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const long long v = e / C;
        const int w = (int)(v % df.W), h = (int)((v / df.W) % df.H), d = (int)((v / ((long long)df.W * df.H)) % df.D);
        const long long n = v / ((long long)df.W * df.H * df.D);
        const long long vl = ((n * (df.D / 2) + d / 2) * (df.H / 2) + h / 2) * (df.W / 2) + w / 2;
        gf[e] += gc[vl * C + c] * 0.125f;
    }
}

// g16 = g32 * (y > 0) (ReLU backward) in BF16; y == nullptr: no mask.
__global__ void k_relu_bwd(const float* __restrict__ g32, const bf16* __restrict__ y, bf16* __restrict__ g16,
                           long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        float gv = g32[e];
        if (y && !(__bfloat162float(y[e]) > 0.f)) gv = 0.f;
        g16[e] = __float2bfloat16(gv);
    }
}

// Weighted mean-squared loss over the first OC channels of out (C channels
// per voxel): g[v][c] = 2 w (out - t) / (OC V) for c < OC, else 0; w times
// the mean square added to *loss.
__global__ void k_mse(const float* __restrict__ out, const float* __restrict__ t, float* __restrict__ g, long long V,
                      int C, int OC, float w, double* __restrict__ loss) {
    double s = 0.0;
    const float sc = 2.f * w / (float)(OC * V);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < V * C; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const long long v = e / C;
        float gv = 0.f;
        if (c < OC) {
            const float d = out[e] - t[v * OC + c];
            s += (double)d * d;
            gv = sc * d;
        }
        g[e] = gv;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(loss, (double)w * s / (double)(OC * V));
}

// Adam (Kingma & Ba 2015) with bias correction; c1 = lr / (1 - b1^t),
// c2 = 1 / (1 - b2^t).
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, float b1, float b2, float eps, float c1, float c2) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float gv = g[e];
        const float mv = b1 * m[e] + (1.f - b1) * gv;
        const float vv = b2 * v[e] + (1.f - b2) * gv * gv;
        m[e] = mv;
        v[e] = vv;
        p[e] -= c1 * mv / (sqrtf(vv * c2) + eps);
    }
}

// BF16 copies of one layer's weights: forward Wk[tap][co][ci] and the
// flipped, transposed kernel of the input gradient Wt[26 - tap][ci][co].
__global__ void k_weights_bf16(const float* __restrict__ W, bf16* __restrict__ Wk, bf16* __restrict__ Wt, int cin,
                               int cout) {
    const int n = 27 * cin * cout;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int ci = e % cin, co = (e / cin) % cout, tap = e / (cin * cout);
        const bf16 b = __float2bfloat16(W[e]);
        Wk[e] = b;
        Wt[((size_t)(26 - tap) * cin + ci) * cout + co] = b;
    }
}

}  // namespace nn
}  // namespace pic
