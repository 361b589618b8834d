// krylov.cuh -- FP64 vector kernels of the GMRES family: deterministic
// block-partial dot products (fixed grid, fixed-order final sum), batched
// dots for classical Gram-Schmidt, and axpy-type updates whose scalars stay
// in device memory so an Arnoldi step needs no host round trip.
#pragma once
#include "common.cuh"

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

// flag[0] |= any non-finite value
__global__ void k_nonfinite(const double* __restrict__ a, long long n, int* __restrict__ flag) {
    int bad = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (!isfinite(a[i])) bad = 1;
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

}  // namespace pic
