// nn_kernels.cuh -- kernels of the learned preconditioner's network besides
// the tensor-core convolution (conv_tc.cuh): pooling / upsampling / skip
// concatenation, their backward passes, weight gradients, the loss and Adam.
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
    // one thread per (coarse voxel, 8-channel chunk): 16-byte loads and stores, 32-bit index math
    const int D2 = di.D / 2, H2 = di.H / 2, W2 = di.W / 2, C8 = C / 8;
    const int tot = di.N * D2 * H2 * W2 * C8;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
        const int c8 = e % C8, v = e / C8;
        const int w = v % W2, h = (v / W2) % H2, d = (v / (W2 * H2)) % D2, n = v / (W2 * H2 * D2);
        float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int dd = 2 * d + (q >> 2), hh = 2 * h + ((q >> 1) & 1), ww = 2 * w + (q & 1);
            const uint4 u = *reinterpret_cast<const uint4*>(
                x + ((((long long)n * di.D + dd) * di.H + hh) * di.W + ww) * C + c8 * 8);
            const __nv_bfloat162* p2 = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float2 f = __bfloat1622float2(p2[i]);
                s[2 * i] += f.x;
                s[2 * i + 1] += f.y;
            }
        }
        __align__(16) __nv_bfloat162 o[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) o[i] = __floats2bfloat162_rn(s[2 * i] * 0.125f, s[2 * i + 1] * 0.125f);
        *reinterpret_cast<uint4*>(y + (long long)v * C + c8 * 8) = *reinterpret_cast<const uint4*>(o);
    }
}

// y[v] = concat(lo[v / 2] (C1 channels, nearest upsampling), skip[v] (C2)),
// dims of the fine level.  One thread per (voxel, 8-channel chunk).
__global__ void k_up_concat(const bf16* __restrict__ lo, const bf16* __restrict__ skip, bf16* __restrict__ y, Dims df,
                            int C1, int C2) {
    const int C8 = (C1 + C2) / 8, L8 = C1 / 8;
    const int tot = (int)df.vox() * C8;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
        const int c8 = e % C8, v = e / C8;
        uint4 u;
        if (c8 >= L8) {
            u = *reinterpret_cast<const uint4*>(skip + (long long)v * C2 + (c8 - L8) * 8);
        } else {
            const int w = v % df.W, h = (v / df.W) % df.H, d = (v / (df.W * df.H)) % df.D, n = v / (df.W * df.H * df.D);
            const long long vl = (((long long)n * (df.D / 2) + d / 2) * (df.H / 2) + h / 2) * (df.W / 2) + w / 2;
            u = *reinterpret_cast<const uint4*>(lo + vl * C1 + c8 * 8);
        }
        *reinterpret_cast<uint4*>(y + (long long)e * 8) = u;
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
