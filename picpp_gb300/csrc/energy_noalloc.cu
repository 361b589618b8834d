// energy_noalloc.cu -- pic_energy_noalloc: the energy and momentum sums of
// pic_energy for device arrays the caller owns, without allocating anything.
//
// Who needs it: callers that may not allocate device memory at the point
// where they want the diagnostics -- hosts that hand the GPU to a fixed
// memory pool at start-up and forbid allocations afterwards, and embedders
// whose device memory comes from their own allocator rather than the CUDA
// runtime's.  They keep E, B and the momenta in their own buffers and pass
// device pointers in.  The call copies the six sums to the caller's host
// array and synchronises the given stream before it returns.
//
// Scratch: the reduction partial sums live in one file-scope device array,
// g_energy_scratch (548,864 bytes, 67 rows of 1024 doubles), which every GPU
// that loads the library holds until the process exits.  Every call reuses
// it, so two calls that overlap on the GPU (different streams, no ordering
// between them) race on it.  Each call overwrites every partial it reads
// before reading it, so nothing has to be cleared between calls.
//
// Host code cannot use &g_energy_scratch as a device address (the host-side
// symbol is only a stand-in).  The first call on a device looks the device
// address up with cudaGetSymbolAddress while that device is current and
// caches it (the lookup may initialise the module).  cudaDeviceReset unloads the module,
// so the cached address is not valid after a reset: do not call this entry
// point on a device that was reset since its first call.
#include <cmath>
#include <mutex>

#include "../../include/picpp_gb300.h"
#include "common.cuh"

namespace {

constexpr int kBlocks = 1024;                   // partials per reduction row
constexpr int kMaxSpecies = PIC_NOALLOC_MAX_SPECIES;
constexpr int kRows = 4 * kMaxSpecies + 3;      // 4 sums per species, E^2, B^2, results

__device__ __align__(256) double g_energy_scratch[kRows * kBlocks];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {};

using pic::block_sum;
using pic::kRedThreads;

// Kinetic energy and momentum partials of one species into rows 4s..4s+3.
__global__ void __launch_bounds__(kRedThreads) k_na_particles(const double* __restrict__ px, const double* __restrict__ py,
                                                              const double* __restrict__ pz, long long n, double m,
                                                              double w, double* __restrict__ rows, int P) {
    __shared__ double sh[32];
    double s[4] = {0, 0, 0, 0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double a = px[i], b = py[i], c = pz[i];
        double gam = sqrt((a * a + b * b + c * c) / (m * m) + 1.0);
        s[0] += (gam - 1) * m * w;
        s[1] += a * w; s[2] += b * w; s[3] += c * w;
    }
    for (int q = 0; q < 4; ++q) {
        double r = block_sum(s[q], sh);
        if (threadIdx.x == 0) rows[q * kBlocks + blockIdx.x] = r;
    }
}

__global__ void __launch_bounds__(kRedThreads) k_na_squares(const double* __restrict__ a, long long n,
                                                            double* __restrict__ row) {
    __shared__ double sh[32];
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += a[i] * a[i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) row[blockIdx.x] = s;
}

// One block per output k = 0..5 (kinetic, E, B, px, py, pz): the fixed-order
// sum of that quantity's partial rows, written to the results row.
__global__ void k_na_finalize(const double* __restrict__ scratch, int nspecies, int Pp, int Pf, double field_scale,
                              double* __restrict__ result) {
    __shared__ double sh[32];
    const int k = blockIdx.x;   // 0..5
    double s = 0.0;
    if (k == 1 || k == 2) {
        const double* row = scratch + (4 * kMaxSpecies + (k - 1)) * kBlocks;
        for (int i = threadIdx.x; i < Pf; i += blockDim.x) s += row[i];
    } else {
        const int q = k == 0 ? 0 : k - 2;   // out index -> per-species row
        for (int sp = 0; sp < nspecies; ++sp) {
            const double* row = scratch + (4 * sp + q) * kBlocks;
            double t = 0.0;
            for (int i = threadIdx.x; i < Pp; i += blockDim.x) t += row[i];
            s += t;
        }
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) result[k] = (k == 1 || k == 2) ? s * field_scale : s;
}

pic_status scratch_for_current_device(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PIC_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_energy_scratch);
        if (e != cudaSuccess || p == nullptr) return PIC_ERR_CUDA;
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_ptr[dev];
    return PIC_OK;
}

int blocks_for(long long n) {
    long long b = (n + kRedThreads - 1) / kRedThreads;
    if (b > kBlocks) b = kBlocks;
    if (b < 1) b = 1;
    return (int)b;
}

}  // namespace

extern "C" pic_status pic_energy_noalloc(int nx, int ny, int nz, double dx, double dy, double dz, const double* E,
                                         const double* B, int nspecies, const long* counts, const double* masses,
                                         const double* weights, const double* const* px, const double* const* py,
                                         const double* const* pz, void* stream, double out[6]) {
    if (nx < 1 || ny < 1 || nz < 1 || !(dx > 0) || !(dy > 0) || !(dz > 0) || !out) return PIC_ERR_ARG;
    if ((long long)nx * ny * nz >= (1LL << 31)) return PIC_ERR_ARG;
    if (nspecies < 0 || nspecies > kMaxSpecies) return PIC_ERR_ARG;   // rows for at most 16 species
    if (nspecies > 0 && (!counts || !masses || !weights || !px || !py || !pz)) return PIC_ERR_ARG;
    for (int s = 0; s < nspecies; ++s) {
        if (counts[s] < 0 || !(masses[s] > 0)) return PIC_ERR_ARG;
        if (counts[s] > 0 && (!px[s] || !py[s] || !pz[s])) return PIC_ERR_ARG;
    }
    double* scratch = nullptr;
    pic_status st = scratch_for_current_device(&scratch);
    if (st != PIC_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long L = 3LL * nx * ny * nz;
    int Pp = 1;
    for (int sp = 0; sp < nspecies; ++sp) {
        const int P = blocks_for(counts[sp]);
        Pp = P > Pp ? P : Pp;
    }
    // every species writes Pp partials per row so the finalisation reads
    // only values written by this call
    for (int sp = 0; sp < nspecies; ++sp)
        k_na_particles<<<Pp, kRedThreads, 0, s>>>(px[sp], py[sp], pz[sp], counts[sp], masses[sp], weights[sp],
                                                  scratch + 4 * sp * kBlocks, Pp);
    const int Pf = blocks_for(L);
    k_na_squares<<<Pf, kRedThreads, 0, s>>>(E, E ? L : 0, scratch + (4 * kMaxSpecies) * kBlocks);
    k_na_squares<<<Pf, kRedThreads, 0, s>>>(B, B ? L : 0, scratch + (4 * kMaxSpecies + 1) * kBlocks);
    const double scale = dx * dy * dz / (8 * 3.14159265358979323846);
    double* result = scratch + (kRows - 1) * kBlocks;   // the results row
    k_na_finalize<<<6, kRedThreads, 0, s>>>(scratch, nspecies, Pp, Pf, scale, result);
    if (cudaGetLastError() != cudaSuccess) return PIC_ERR_CUDA;
    if (cudaMemcpyAsync(out, result, 6 * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) return PIC_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return PIC_ERR_CUDA;
    return PIC_OK;
}
