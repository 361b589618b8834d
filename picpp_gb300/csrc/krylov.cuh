// krylov.cuh -- FP64 vector kernels of the GMRES family: deterministic
// block-partial dot products (fixed grid, fixed-order final sum), batched
// dots for classical Gram-Schmidt, and axpy-type updates whose scalars stay
// in device memory so an Arnoldi step needs no host round trip.
#pragma once
#include "common.cuh"
#include "kernels.hpp"

namespace pic {

// partials[blockIdx.x] = sum over this block's grid-stride slice of a*b.
__global__ void __launch_bounds__(kRedThreads) k_dot_partials(const double* __restrict__ a, const double* __restrict__ b,
                                                              long long n, double* __restrict__ partials) {
    __shared__ double sh[32];
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += a[i] * b[i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// Batched dots of w against k basis vectors V[m] (stride ld): partials[m*P + block].
template <int KB>
__global__ void __launch_bounds__(kRedThreads) k_multi_dot_partials(const double* __restrict__ V, long long ld, int k0, int k,
                                                                    const double* __restrict__ w, long long n,
                                                                    double* __restrict__ partials, int P) {
    __shared__ double sh[32];
    double acc[KB];
#pragma unroll
    for (int m = 0; m < KB; ++m) acc[m] = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double wi = w[i];
#pragma unroll
        for (int m = 0; m < KB; ++m)
            if (k0 + m < k) acc[m] += V[(long long)(k0 + m) * ld + i] * wi;
    }
#pragma unroll
    for (int m = 0; m < KB; ++m) {
        if (k0 + m >= k) break;
        double s = block_sum(acc[m], sh);
        if (threadIdx.x == 0) partials[(long long)(k0 + m) * P + blockIdx.x] = s;
    }
}

// out[m * ostride] = sum of partials[m*P .. m*P+P) in a fixed tree order
// (optionally sqrt).  One block per vector.
__global__ void __launch_bounds__(kRedThreads) k_finalize(const double* __restrict__ partials, int P, double* __restrict__ out,
                                                          int ostride, int take_sqrt) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int i = threadIdx.x; i < P; i += blockDim.x) s += partials[(long long)blockIdx.x * P + i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[(long long)blockIdx.x * ostride] = take_sqrt ? sqrt(s) : s;
}

// y -= alpha[0] * x, alpha in device memory.
__global__ void k_axpy_minus_dev(double* __restrict__ y, const double* __restrict__ x, const double* __restrict__ alpha,
                                 long long n) {
    const double a = *alpha;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] -= a * x[i];
}

// w -= sum_m h[m * hstride] V[m], m < k (classical Gram-Schmidt update).
__global__ void k_multi_axpy_minus(double* __restrict__ w, const double* __restrict__ V, long long ld, int k,
                                   const double* __restrict__ h, int hstride, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double s = w[i];
        for (int m = 0; m < k; ++m) s -= h[m * hstride] * V[(long long)m * ld + i];
        w[i] = s;
    }
}

// v = w / h[0] (v = 0 when h[0] == 0, specialmath.cpp:336-349).
__global__ void k_scale_inv_dev(double* __restrict__ v, const double* __restrict__ w, const double* __restrict__ h,
                                long long n) {
    // one reciprocal per thread: an FP64 division per element would make
    // this copy arithmetic-bound on this GPU's FP64 pipe
    const double d = *h;
    const double inv = d > 0 ? 1.0 / d : 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[i] = w[i] * inv;
}

// v = w * s (host scalar)
__global__ void k_scale(double* __restrict__ v, const double* __restrict__ w, double s, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[i] = w[i] * s;
}

// v = w / s (host scalar), exact division.
__global__ void k_div(double* __restrict__ v, const double* __restrict__ w, double s, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[i] = w[i] / s;
}

// x (+)= sum_m V[m] * y[m] * scale, m in order (specialmath.cpp:625-634).
__global__ void k_combine(double* __restrict__ x, const double* __restrict__ V, long long ld, int k,
                          const double* __restrict__ y, double scale, int accumulate, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double s = accumulate ? x[i] : 0.0;
        for (int m = 0; m < k; ++m) s += V[(long long)m * ld + i] * y[m] * scale;
        x[i] = s;
    }
}

// r = b - Ax
__global__ void k_residual(double* __restrict__ r, const double* __restrict__ b, const double* __restrict__ Ax, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        r[i] = b[i] - Ax[i];
}

// ---- FP32 vectors of the mixed-precision preconditioner's inner solve:
// products accumulated in FP32 per thread and in FP64 across threads,
// Hessenberg entries and coefficients kept in FP64.  Each reduction is one
// launch: every block writes its partial sums, and the last block to finish
// (a global counter) adds all partials in a fixed order, so the result does
// not depend on the order in which blocks ran.

// True in the block that finished last (counter reset for the next launch
// by that block's caller after its final sums).
__device__ __forceinline__ bool last_block(unsigned* counter) {
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    return is_last;
}

// out[m] = sum of partials[m * P .. m * P + P), m in [m0, m1), fixed order
// (run by the last block; partials read around L1).
__device__ __forceinline__ void finalize_rows(const double* partials, int P, int m0, int m1, double* out,
                                              double* sh) {
    for (int m = m0; m < m1; ++m) {
        double t = 0.0;
        for (int i = threadIdx.x; i < P; i += blockDim.x) t += __ldcg(&partials[(long long)m * P + i]);
        t = block_sum(t, sh);
        if (threadIdx.x == 0) out[m] = t;
    }
}

// Element access of the FP32 kernels: W = 4 reads and writes float4 (the
// vectors' length a multiple of 4 and their bases 16-byte aligned, which the
// launchers check), W = 1 single floats.
template <int W>
struct F32Vec;
template <>
struct F32Vec<1> {
    using T = float;
    static __device__ __forceinline__ float dot(float a, float b, float acc) { return fmaf(a, b, acc); }
    static __device__ __forceinline__ float axpy(float a, float x, float y) { return fmaf(a, x, y); }
    static __device__ __forceinline__ float scale(float x, float f) { return x * f; }
    static __device__ __forceinline__ float zero() { return 0.f; }
};
template <>
struct F32Vec<4> {
    using T = float4;
    static __device__ __forceinline__ float dot(float4 a, float4 b, float acc) {
        return fmaf(a.w, b.w, fmaf(a.z, b.z, fmaf(a.y, b.y, fmaf(a.x, b.x, acc))));
    }
    static __device__ __forceinline__ float4 axpy(float a, float4 x, float4 y) {
        return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
    }
    static __device__ __forceinline__ float4 scale(float4 x, float f) {
        return make_float4(x.x * f, x.y * f, x.z * f, x.w * f);
    }
    static __device__ __forceinline__ float4 zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
};

// out[0] = a . b (FP32 vectors; n counts elements of W floats).
template <int W>
__global__ void __launch_bounds__(kRedThreads) k_dot_f32(const float* __restrict__ a_, const float* __restrict__ b_,
                                                         long long n, double* __restrict__ partials,
                                                         double* __restrict__ out, unsigned* __restrict__ counter) {
    using V = F32Vec<W>;
    const typename V::T* a = reinterpret_cast<const typename V::T*>(a_);
    const typename V::T* b = reinterpret_cast<const typename V::T*>(b_);
    __shared__ double sh[32];
    float s = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s = V::dot(a[i], b[i], s);
    const double t = block_sum(double(s), sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
    if (last_block(counter)) {
        finalize_rows(partials, gridDim.x, 0, 1, out, sh);
        if (threadIdx.x == 0) *counter = 0u;
    }
}

// out[m] = V[m] . w for m in [k0, min(k0 + KB, k)) (FP32 basis, stride ld
// in elements of W floats).
template <int KB, int W>
__global__ void __launch_bounds__(kRedThreads) k_multi_dot_f32(const float* __restrict__ V_, long long ld, int k0,
                                                               int k, const float* __restrict__ w_, long long n,
                                                               double* __restrict__ partials,
                                                               double* __restrict__ out,
                                                               unsigned* __restrict__ counter,
                                                               const unsigned* __restrict__ skip) {
    if (*skip) return;   // the inner solve has converged
    using F = F32Vec<W>;
    const typename F::T* V = reinterpret_cast<const typename F::T*>(V_);
    const typename F::T* w = reinterpret_cast<const typename F::T*>(w_);
    __shared__ double sh[32];
    float acc[KB];
#pragma unroll
    for (int m = 0; m < KB; ++m) acc[m] = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const typename F::T wi = w[i];
#pragma unroll
        for (int m = 0; m < KB; ++m)
            if (k0 + m < k) acc[m] = F::dot(V[(long long)(k0 + m) * ld + i], wi, acc[m]);
    }
    const int P = gridDim.x;
#pragma unroll
    for (int m = 0; m < KB; ++m) {
        if (k0 + m >= k) break;
        const double t = block_sum(double(acc[m]), sh);
        if (threadIdx.x == 0) partials[(long long)(k0 + m) * P + blockIdx.x] = t;
    }
    if (last_block(counter)) {
        finalize_rows(partials, P, k0, k0 + KB < k ? k0 + KB : k, out, sh);
        if (threadIdx.x == 0) *counter = 0u;
    }
}

// w -= sum_m h[m] V[m], m < k; then out[0] = |w|^2 (FP32 vectors, FP64
// coefficients).
template <int W>
__global__ void __launch_bounds__(kRedThreads) k_axpy_norm_f32(float* __restrict__ w_, const float* __restrict__ V_,
                                                               long long ld, int k, const double* __restrict__ h,
                                                               long long n, double* __restrict__ partials,
                                                               double* __restrict__ out,
                                                               unsigned* __restrict__ counter,
                                                               const unsigned* __restrict__ skip) {
    if (*skip) return;
    using F = F32Vec<W>;
    typename F::T* w = reinterpret_cast<typename F::T*>(w_);
    const typename F::T* V = reinterpret_cast<const typename F::T*>(V_);
    __shared__ double sh[32];
    __shared__ float hs[64];
    for (int m = threadIdx.x; m < k; m += blockDim.x) hs[m] = float(h[m]);
    __syncthreads();
    float nrm = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        typename F::T s = w[i];
        for (int m = 0; m < k; ++m) s = F::axpy(-hs[m], V[(long long)m * ld + i], s);
        w[i] = s;
        nrm = F::dot(s, s, nrm);
    }
    const double t = block_sum(double(nrm), sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
    if (last_block(counter)) {
        finalize_rows(partials, gridDim.x, 0, 1, out, sh);
        if (threadIdx.x == 0) *counter = 0u;
    }
}

// v = w / sqrt(h2[0]) (zero for h2[0] <= 0); one square root per block.
template <int W>
__global__ void k_normalize_f32(float* __restrict__ v_, const float* __restrict__ w_, const double* __restrict__ h2,
                                long long n, const unsigned* __restrict__ skip) {
    if (*skip) return;
    using F = F32Vec<W>;
    typename F::T* v = reinterpret_cast<typename F::T*>(v_);
    const typename F::T* w = reinterpret_cast<const typename F::T*>(w_);
    __shared__ float inv;
    if (threadIdx.x == 0) {
        const double d = *h2;
        inv = d > 0 ? float(1.0 / sqrt(d)) : 0.f;
    }
    __syncthreads();
    const float f = inv;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[i] = F::scale(w[i], f);
}

// dst = src (FP64 to FP32).
__global__ void k_to_f32(float* __restrict__ dst, const double* __restrict__ src, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = float(src[i]);
}

// z = scale * sum_m V[m] y[m], m < *kp, in FP64 (FP32 basis, FP64
// coefficients).
__global__ void k_combine_f32(double* __restrict__ z, const float* __restrict__ V, long long ld,
                              const unsigned* __restrict__ kp, const double* __restrict__ y, double scale, long long n) {
    const int k = (int)*kp;
    __shared__ float ys[64];
    for (int m = threadIdx.x; m < k; m += blockDim.x) ys[m] = float(y[m]);
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int m = 0; m < k; ++m) s = fmaf(ys[m], V[(long long)m * ld + i], s);
        z[i] = double(s) * scale;
    }
}

// One Givens step of the inner least-squares problem, on the device (one
// thread): rotates column j with the previous rotations, forms rotation j
// from the column's diagonal and the new vector's norm, updates g and sets
// flags[1] (done) when |g_{j+1}| <= tol |v| or the Krylov space is
// invariant; flags[2] = the columns in use.
__global__ void k_inner_givens(int j, InnerLayout L, double* __restrict__ h, double tol, unsigned* __restrict__ flags) {
    if (threadIdx.x != 0 || flags[1]) return;
    double* col = h + L.h() + (long long)j * (L.S + 1);
    double* cs = h + L.cs();
    double* sn = h + L.sn();
    double* gv = h + L.g();
    if (j == 0) {
        h[1] = sqrt(fmax(h[0], 0.0));
        gv[0] = h[1];
    }
    for (int i = 0; i < j; ++i) {
        const double t = cs[i] * col[i] + sn[i] * col[i + 1];
        col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1];
        col[i] = t;
    }
    const double a = col[j], b = sqrt(fmax(h[L.hn() + j], 0.0));
    const double mod = hypot(a, b);
    const double c_ = mod == 0 ? 1.0 : a / mod, s_ = mod == 0 ? 0.0 : b / mod;
    cs[j] = c_;
    sn[j] = s_;
    col[j] = mod;
    gv[j + 1] = -s_ * gv[j];
    gv[j] = c_ * gv[j];
    flags[2] = (unsigned)(j + 1);
    if (!(b > 0) || fabs(gv[j + 1]) <= tol * h[1]) flags[1] = 1u;
}

// y = R^{-1} g over the flags[2] columns in use (one thread); clears the
// done flag for the next solve.
__global__ void k_inner_backsolve(InnerLayout L, double* __restrict__ h, unsigned* __restrict__ flags) {
    if (threadIdx.x != 0) return;
    const int kk = (int)flags[2];
    double* y = h + L.y();
    const double* gv = h + L.g();
    for (int i = kk - 1; i >= 0; --i) {
        double acc = gv[i];
        for (int q = i + 1; q < kk; ++q) acc -= h[L.h() + (long long)q * (L.S + 1) + i] * y[q];
        const double d = h[L.h() + (long long)i * (L.S + 1) + i];
        y[i] = d != 0 ? acc / d : 0.0;
    }
    flags[1] = 0u;
}

// flag[0] |= any non-finite value
__global__ void k_nonfinite(const double* __restrict__ a, long long n, int* __restrict__ flag) {
    int bad = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (!isfinite(a[i])) bad = 1;
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

}  // namespace pic
