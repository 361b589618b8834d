// common.cuh -- shared device helpers of the GB300 PIC hot path.
//
// Grid conventions: periodic box, arrays a[c][k][j][i] with i fastest; node
// (i,j,k) at (i dx, j dy, k dz), cell (i,j,k) spanning [i dx, (i+1) dx) ...
// Particles: linear cell index + in-cell offsets in [0,1) + momentum.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pic {

// Division of non-negative ints below 2^31 by a fixed divisor with a multiply
// and a shift (Granlund & Montgomery, PLDI 1994): q = (umulhi(m, n) + n) >> l.
struct FastDiv {
    unsigned m = 1, l = 0;
    FastDiv() = default;
    explicit FastDiv(unsigned d) {
        l = 0;
        while ((1u << l) < d) ++l;
        m = (unsigned)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    }
};

struct GridP {
    int nx, ny, nz;
    int wall;             // 1: conductor wall at x = 0, open boundary at x = (nx - 2) dx (wall.cuh)
    long long N;          // nx*ny*nz
    double dx, dy, dz, dt;
    double idx, idy, idz; // 1/dx ...
    double theta, eta, cfix;
    int y3, z3;           // ny > 1, nz > 1
    FastDiv divx, divy;   // by nx, by ny
};
// The explicit (Tristan) mover of a wall box reflects at
// xgrid[reflectingWallPoint] (mover.cpp:746-750; reflectingWallPoint = 20
// in the reference's ghosted index, constants.h:64): node 18 here, two
// ghost layers left of node 0.
constexpr int kTristanWallNode = 18;

// 128 bytes: the size up to which the out-of-line gathers take it in
// registers (a larger struct goes through a stack frame)
static_assert(sizeof(GridP) == 128, "GridP layout");

__device__ __forceinline__ int fast_div(int n, const FastDiv& f) {
    return (int)((__umulhi(f.m, (unsigned)n) + (unsigned)n) >> f.l);
}

__host__ __device__ __forceinline__ int wrap_p(int a, int n) { return a >= n ? a - n : a; }
__host__ __device__ __forceinline__ int wrap_m(int a, int n) { return a < 0 ? a + n : a; }
__host__ __device__ __forceinline__ int wrap_any(int a, int n) { a %= n; return a < 0 ? a + n : a; }

__host__ __device__ __forceinline__ long long lin(const GridP& g, int i, int j, int k) {
    return ((long long)k * g.ny + j) * g.nx + i;
}
// Linear index with a periodic wrap of offsets in [-n, 2n).
__host__ __device__ __forceinline__ long long linw(const GridP& g, int i, int j, int k) {
    i = i < 0 ? i + g.nx : (i >= g.nx ? i - g.nx : i);
    j = j < 0 ? j + g.ny : (j >= g.ny ? j - g.ny : j);
    k = k < 0 ? k + g.nz : (k >= g.nz ? k - g.nz : k);
    return ((long long)k * g.ny + j) * g.nx + i;
}
__host__ __device__ __forceinline__ void decode(const GridP& g, int cell, int& i, int& j, int& k) {
#ifdef __CUDA_ARCH__
    int q = fast_div(cell, g.divx);
    i = cell - q * g.nx;
    k = fast_div(q, g.divy);
    j = q - k * g.ny;
#else
    int q = cell / g.nx;
    i = cell - q * g.nx;
    k = q / g.ny;
    j = q - k * g.ny;
#endif
}

// Division that is exact in FP64 (to match the oracle operation by
// operation) and a reciprocal multiply in FP32 (tolerance-checked path).
template <typename T> __device__ __forceinline__ T divd(T a, T d, T invd);
template <> __device__ __forceinline__ double divd<double>(double a, double d, double) { return a / d; }
template <> __device__ __forceinline__ float divd<float>(float a, float, float invd) { return a * invd; }

template <typename T> __device__ __forceinline__ T dev_sqrt(T x);
template <> __device__ __forceinline__ double dev_sqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float dev_sqrt<float>(float x) { return sqrtf(x); }

template <typename T> __device__ __forceinline__ T dev_floor(T x);
template <> __device__ __forceinline__ double dev_floor<double>(double x) { return floor(x); }
template <> __device__ __forceinline__ float dev_floor<float>(float x) { return floorf(x); }

// Asynchronous global -> shared copies of 4 or 8 bytes (cp.async, no
// registers held while in flight); the wait covers the copies the calling
// thread started.
template <int B>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (B == 4) asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Particle state of one species, SoA in device memory.
template <typename T>
struct PartView {
    int* cell;
    T *ox, *oy, *oz, *px, *py, *pz;
    int* id;
    long long n;
};

// Linear weights between the two nearest nodes / cell centres, the
// top-hat overlap the reference computes in correlationBspline case 0
// (PIC++/correlation.cpp:798-836; Yee form correlation.cpp:471-496).
template <typename T>
__device__ __forceinline__ void node_w(T u, int c, int n, int idx[2], T w[2]) {
    if (n == 1) { idx[0] = idx[1] = 0; w[0] = T(1); w[1] = T(0); return; }
    T wl, wr;
    if (u < T(0.5)) { wl = T(0.5) + (T(0.5) - u); wr = T(1) - wl; }
    else            { wr = T(0.5) + (u - T(0.5)); wl = T(1) - wr; }
    idx[0] = c; idx[1] = wrap_p(c + 1, n); w[0] = wl; w[1] = wr;
}
template <typename T>
__device__ __forceinline__ void cell_w(T u, int c, int n, int idx[2], T w[2]) {
    if (n == 1) { idx[0] = idx[1] = 0; w[0] = T(1); w[1] = T(0); return; }
    T wl, wr;
    if (u < T(0.5)) { wr = T(0.5) + u; wl = T(1) - wr; idx[0] = wrap_m(c - 1, n); idx[1] = c; }
    else            { wl = T(0.5) + (T(1) - u); wr = T(1) - wl; idx[0] = c; idx[1] = wrap_p(c + 1, n); }
    w[0] = wl; w[1] = wr;
}

// Advance an in-cell offset by du cells and wrap the cell index; identical
// rule to the oracle's advance_axis.
template <typename T>
__device__ __forceinline__ void advance_axis(T& u, int& c, T du, int n) {
    T un = u + du;
    T s = dev_floor(un);
    un = un - s;
    int ci = c + (int)s;
    if (un >= T(1)) { un -= T(1); ci += 1; }
    u = un;
    int w = ci < 0 ? ci + n : (ci >= n ? ci - n : ci);
    if ((unsigned)w >= (unsigned)n) w = wrap_any(ci, n);   // moved farther than one box length
    c = w;
}

constexpr int kRedThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum in a fixed order; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double* sh) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    __syncthreads();
    return r;
}

}  // namespace pic
