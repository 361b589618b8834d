// kernels_impl.cuh -- launchers of the particle and Yee kernels for one
// particle precision T; instantiated by kernels_f32.cu and kernels_f64.cu.
#pragma once
#include <algorithm>
#include <cmath>
#include "boris.cuh"
#include "boris_tile.cuh"
#include "diag.cuh"
#include "implicit_particles.cuh"
#include "implicit_tile.cuh"
#include "kernels.hpp"
#include "yee.cuh"

namespace pic {

// kGatherBatch destinations per thread per pass: their permutation entries
// and then their 8 x kGatherBatch payload loads are all in flight together
// (one pass is otherwise two dependent memory latencies for 32 bytes).
constexpr int kGatherBatch = 4;
template <typename T>
__global__ void k_gather_payload(const int* __restrict__ perm, long long n, PartView<T> src, PartView<T> dst) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long d0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; d0 < n; d0 += stride * kGatherBatch) {
        int s[kGatherBatch];
#pragma unroll
        for (int k = 0; k < kGatherBatch; ++k) {
            const long long d = d0 + k * stride;
            s[k] = d < n ? perm[d] : -1;
        }
        int cell[kGatherBatch], id[kGatherBatch];
        T v[6][kGatherBatch];
#pragma unroll
        for (int k = 0; k < kGatherBatch; ++k) {
            if (s[k] < 0) continue;
            cell[k] = src.cell[s[k]]; id[k] = src.id[s[k]];
            v[0][k] = src.ox[s[k]]; v[1][k] = src.oy[s[k]]; v[2][k] = src.oz[s[k]];
            v[3][k] = src.px[s[k]]; v[4][k] = src.py[s[k]]; v[5][k] = src.pz[s[k]];
        }
#pragma unroll
        for (int k = 0; k < kGatherBatch; ++k) {
            if (s[k] < 0) continue;
            const long long d = d0 + k * stride;
            dst.cell[d] = cell[k]; dst.id[d] = id[k];
            dst.ox[d] = v[0][k]; dst.oy[d] = v[1][k]; dst.oz[d] = v[2][k];
            dst.px[d] = v[3][k]; dst.py[d] = v[4][k]; dst.pz[d] = v[5][k];
        }
    }
}

// Kinetic energy and momentum of one species: partials[q*P + block],
// q = 0: sum w (gamma - 1) m, 1..3: sum w p (updateEnergy,
// PIC++/simulation.cpp:1590-1600).
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_particle_sums(PartView<T> p, double m, double w, double* __restrict__ partials,
                                                               int P) {
    __shared__ double sh[32];
    double s[4] = {0, 0, 0, 0};
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < p.n; n += (long long)gridDim.x * blockDim.x) {
        double px = p.px[n], py = p.py[n], pz = p.pz[n];
        double p2 = px * px + py * py + pz * pz;
        double gam = sqrt(p2 / (m * m) + 1.0);
        s[0] += (gam - 1) * m * w;
        s[1] += px * w; s[2] += py * w; s[3] += pz * w;
    }
    for (int q = 0; q < 4; ++q) {
        double r = block_sum(s[q], sh);
        if (threadIdx.x == 0) partials[q * P + blockIdx.x] = r;
    }
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_sq_partials(const T* __restrict__ a, long long n, double* __restrict__ partials) {
    __shared__ double sh[32];
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double v = double(a[i]);
        s += v * v;
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

template <typename T>
__global__ void k_convert(const double* __restrict__ s, T* __restrict__ d, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = T(s[i]);
}
// FP64 host values to the particle precision with the range checks of
// k_validate done on the FP64 values: mode 0 in-cell offsets (must lie in
// [0,1); an offset that rounds up to 1 in T is kept just below 1), mode 1
// momenta (must be finite).
template <typename T>
__global__ void k_convert_checked(const double* __restrict__ s, T* __restrict__ d, long long n, int mode,
                                  int* __restrict__ flag) {
    int bad = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double v = s[i];
        T t = T(v);
        if (mode == 0) {
            if (!(v >= 0.0 && v < 1.0)) bad |= 2;
            if (t >= T(1)) t = T(1) - T(1) / T(1 << 24);   // largest float below 1 (0.99999994)
        } else if (!isfinite(v)) {
            bad |= 4;
        }
        d[i] = t;
    }
    if (bad) atomicOr(flag, bad);
}

template <typename T>
__global__ void k_convert_back(const T* __restrict__ s, double* __restrict__ d, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = double(s[i]);
}

// flag bits: 1 cell out of range, 2 offset outside [0,1), 4 non-finite momentum
template <typename T>
__global__ void k_validate(GridP g, PartView<T> p, int* __restrict__ flag) {
    int bad = 0;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < p.n; n += (long long)gridDim.x * blockDim.x) {
        int c = p.cell[n];
        if (c < 0 || c >= g.N) bad |= 1;
        else if (g.wall && c % g.nx >= g.nx - 2) bad |= 1;   // wall box: the two ghost columns hold no particles
        T o[3] = {p.ox[n], p.oy[n], p.oz[n]};
        for (int a = 0; a < 3; ++a)
            if (!(o[a] >= T(0) && o[a] < T(1))) bad |= 2;
        T m[3] = {p.px[n], p.py[n], p.pz[n]};
        for (int a = 0; a < 3; ++a)
            if (!isfinite(m[a])) bad |= 4;
    }
    if (bad) atomicOr(flag, bad);
}

template <typename T>
__global__ void k_iota(int* __restrict__ a, long long n, long long start) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        a[i] = (int)(start + i);
}

template <typename T>
void PK<T>::validate(cudaStream_t s, const GridP& g, PartView<T> p, int* flag) {
    if (p.n == 0) return;
    k_validate<T><<<grid_for(p.n, 256, 16), 256, 0, s>>>(g, p, flag);
}

template <typename T>
void PK<T>::iota(cudaStream_t s, int* a, long long n, long long start) {
    if (n == 0) return;
    k_iota<T><<<grid_for(n, 256, 16), 256, 0, s>>>(a, n, start);
}

template <typename T>
void PK<T>::yee_b_half(cudaStream_t s, const GridP& g, void* E, void* B) {
    const T cdtd2 = T(g.cfix * g.dt / 2.0);
    if (g.wall) k_wall_yee_ghosts<T><<<grid_for((long long)g.ny * g.nz, 128), 128, 0, s>>>(g, (T*)E, (T*)B);
    k_yee_b_half<T><<<grid_for(g.N, 256), 256, 0, s>>>(g, (const T*)E, (T*)B, cdtd2, T(g.dx), T(g.dy), T(g.dz),
                                                      T(g.idx), T(g.idy), T(g.idz));
}

template <typename T>
void PK<T>::yee_e(cudaStream_t s, const GridP& g, void* E, const void* B, const double* J, const double er[3]) {
    k_yee_e<T><<<grid_for(g.N, 256), 256, 0, s>>>(g, (T*)E, (const T*)B, J, T(g.cfix), T(g.dt), T(g.dx), T(g.dy),
                                                 T(g.dz), T(g.idx), T(g.idy), T(g.idz), T(er[1]), T(er[2]));
}

template <typename T>
void PK<T>::boris_push(cudaStream_t s, const GridP& g, PartView<T> p, double q, double m, const void* E, const void* B) {
    if (p.n == 0) return;
    k_boris_push<T, T><<<grid_for(p.n, 256, 32), 256, 0, s>>>(g, p, T(q), T(m), (const T*)E, (const T*)B);
}

template <typename T>
void PK<T>::zigzag(cudaStream_t s, const GridP& g, PartView<T> p, double q, double m, double w, double* J) {
    if (p.n == 0) return;
    k_zigzag<T><<<grid_for(p.n, 256, 32), 256, 0, s>>>(g, p, T(q), T(m), T(w), J);
}

template <typename T>
size_t PK<T>::tile_smem_bytes(const TileShape& sh) {
    size_t F = (size_t)sh.fx * sh.fy * sh.fz;
    // FP32: the current block is 64-bit fixed point in two 32-bit words,
    // followed by the warps' scratch for spreading the run heads' adds
    const size_t fixed_scratch = sizeof(T) == 4 ? (size_t)(kTileThreads / 32) * kSpreadBytes : 0;
    // and every warp's staged chunk of particles
    return ((6 * F * sizeof(T) + 15) & ~size_t(15)) + ((3 * (size_t)sh.jcells * 8 + 15) & ~size_t(15)) + fixed_scratch +
           (size_t)(kTileThreads / 32) * sizeof(ChunkBuf<T>);
}

template <typename T>
void PK<T>::push_deposit_tiled(cudaStream_t s, const GridP& g, const TileGeom& t, const TileShape& sh,
                               const SpeciesSet<T>& S, const void* E, const void* B, double* Jpart, double* Jfix,
                               int grid, size_t smem) {
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_push_deposit_tile<T, T, 8, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_push_deposit_tile<T, T, 0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_push_deposit_tile<T, T, 0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    const bool cube8 = t.tx == 8 && t.ty == 8 && t.tz == 8 && g.y3 && g.z3 && sh.fx == 12 && sh.fy == 12 &&
                       sh.fz == 12 && sh.jx == 12 && sh.jy == 12 && sh.jz == 12;
    const float fx_scale = fixed_scale(g, S);
    const double inv_dt = 1.0 / g.dt;
    // a wall box runs its own instantiation (run-time tile shape)
    if (g.wall)
        k_push_deposit_tile<T, T, 0, true><<<grid, kTileThreads, smem, s>>>(g, t, sh, S, (const T*)E, (const T*)B, Jpart,
                                                                           fx_scale, inv_dt);
    else if (cube8)
        k_push_deposit_tile<T, T, 8, false><<<grid, kTileThreads, smem, s>>>(g, t, sh, S, (const T*)E, (const T*)B, Jpart,
                                                                            fx_scale, inv_dt);
    else
        k_push_deposit_tile<T, T, 0, false><<<grid, kTileThreads, smem, s>>>(g, t, sh, S, (const T*)E, (const T*)B, Jpart,
                                                                            fx_scale, inv_dt);
    // the particles it left over: one thread per mask word
    long long words = 1;
    for (int q = 0; q < S.ns; ++q) words = std::max(words, (S.p[q].n + 31) / 32 + 1);
    k_push_deposit_deferred<T, T><<<grid_for(words, 256), 256, 0, s>>>(g, S, (const T*)E, (const T*)B, Jfix);
}

// Fixed-point scale of the FP32 current block: the power of two with
// max_species |q w / V| * scale <= 2^35 (every zigzag term is bounded by
// q w / V because |v| < c = 1, so a run total of up to 32 terms stays below
// 2^40; a tile entry takes at most two terms per particle of the tile, and
// a cell's sum of at most 27 tile partials stays below 2^63 up to about five
// million particles per tile).
template <typename T>
float PK<T>::fixed_scale(const GridP& g, const SpeciesSet<T>& S) {
    double fmax = 0;
    for (int q = 0; q < S.ns; ++q)
        fmax = std::max(fmax, std::fabs((double)S.q[q] * (double)S.w[q] / (g.dx * g.dy * g.dz)));
    return fmax > 0 ? (float)std::ldexp(1.0, 35 - (int)std::ceil(std::log2(fmax))) : 1.0f;
}

template <typename T>
void PK<T>::assemble_j(cudaStream_t s, const GridP& g, const TileGeom& t, const TileShape& sh, const double* Jpart,
                       const double* Jfix, double* J, double inv_scale) {
    k_assemble_j<T><<<grid_for(g.N, 256), 256, 0, s>>>(g, t, sh, Jpart, Jfix, J, inv_scale);
}

template <typename T>
void PK<T>::implicit_deposit(cudaStream_t s, const GridP& g, PartView<T> p, double q, double m, double w,
                             const double* E, const double* B, double* J, double* mu, double* rho, double* Pi,
                             int compat, const GhostAxes& ga) {
    if (p.n == 0) return;
    k_implicit_deposit<T><<<grid_for(p.n, 128, 32), 128, 0, s>>>(g, p, q, m, w, E, B, J, mu, rho, Pi, compat, ga);
}

template <typename T>
ImpBlock PK<T>::implicit_block(const GridP& g, const TileGeom& t, int h) {
    ImpBlock b{};
    b.h = h;
    b.nbx = g.nx > 1 ? t.tx + 2 * h + 1 : 1;
    b.nby = g.y3 ? t.ty + 2 * h + 1 : 1;
    b.nbz = g.z3 ? t.tz + 2 * h + 1 : 1;
    b.cbx = g.nx > 1 ? t.tx + 2 * h + 2 : 1;
    b.cby = g.y3 ? t.ty + 2 * h + 2 : 1;
    b.cbz = g.z3 ? t.tz + 2 * h + 2 : 1;
    b.NB = b.nbx * b.nby * b.nbz;
    b.CB = b.cbx * b.cby * b.cbz;
    return b;
}

template <typename T>
size_t PK<T>::implicit_tile_smem(const ImpBlock& bk) {
    // FP32 accumulators add the per-warp rows of the tensor-core run sums
    // and their 32-entry lane table
    const size_t scratch = sizeof(T) == sizeof(float)
                               ? (size_t)(imp_threads<T>() / 32) * kScrParticles * kScrRow * sizeof(float) + 32 * sizeof(TcLane)
                               : 0;
    return (12 * (size_t)bk.NB + 7 * (size_t)bk.CB + (bk.stage ? 3 * ((size_t)bk.NB + bk.CB) : 0)) * sizeof(T) + scratch;
}

template <typename T>
void PK<T>::implicit_deposit_tiled(cudaStream_t s, const GridP& g, const TileGeom& t, const ImpBlock& bk,
                                   const ImpSpecies<T>& S, const T* E, const T* B, double* J, double* mu,
                                   double* rho, double* Pi) {
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_implicit_deposit_tile<T, T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        cudaFuncSetAttribute(k_implicit_deposit_tile<T, T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        attr_set = true;
    }
    const size_t smem = implicit_tile_smem(bk);
    const int per_sm = (int)((227 * 1024) / (smem + 1024));
    const int ntiles = t.ntx * t.nty * t.ntz;
    const int grid = ntiles < kNumSM * (per_sm > 0 ? per_sm : 1) ? ntiles : kNumSM * (per_sm > 0 ? per_sm : 1);
    constexpr int nt = imp_threads<T>();
    if (bk.stage) k_implicit_deposit_tile<T, T, true><<<grid, nt, smem, s>>>(g, t, bk, S, E, B, J, mu, rho, Pi);
    else k_implicit_deposit_tile<T, T, false><<<grid, nt, smem, s>>>(g, t, bk, S, E, B, J, mu, rho, Pi);
}

template <typename T>
bool PK<T>::implicit_push_tiled(cudaStream_t s, const GridP& g, const TileGeom& t, const ImpSpecies<T>& S,
                                const double* E, const double* B, const double* Et) {
    MoverBlock mb{};
    const int H = kMoverHalo;
    mb.nbx = g.nx > 1 ? t.tx + 2 * H + 1 : 1;
    mb.nby = g.y3 ? t.ty + 2 * H + 1 : 1;
    mb.nbz = g.z3 ? t.tz + 2 * H + 1 : 1;
    mb.cbx = g.nx > 1 ? t.tx + 2 * H + 2 : 1;
    mb.cby = g.y3 ? t.ty + 2 * H + 2 : 1;
    mb.cbz = g.z3 ? t.tz + 2 * H + 2 : 1;
    mb.NB = mb.nbx * mb.nby * mb.nbz;
    mb.CB = mb.cbx * mb.cby * mb.cbz;
    // FP32: E^theta and B^n as float4 nodes / cells, E^n as three planes
    const size_t fld = sizeof(T) == sizeof(float)
                           ? ((size_t)mb.NB + (size_t)mb.CB) * 16 + 3 * (size_t)mb.NB * sizeof(float)
                           : (6 * (size_t)mb.NB + 3 * (size_t)mb.CB) * sizeof(T);
    // plus every thread's staged next particle (6 values and a cell)
    const size_t smem = ((fld + 15) & ~size_t(15)) + (size_t)kMoverThreads * (6 * sizeof(T) + sizeof(int));
    if (smem > 227 * 1024) return false;
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_implicit_push_tile<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        cudaFuncSetAttribute(k_implicit_push_tile<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        attr_set = true;
    }
    const int per_sm = (int)((228 * 1024) / (smem + 1024));
    const int ntiles = t.ntx * t.nty * t.ntz;
    const int cap = kNumSM * (per_sm > 0 ? per_sm : 1);
    // the wall rules are a separate instantiation: the periodic mover keeps
    // none of their code in its loop
    // the particles it left over: one thread per mask word
    long long words = 1;
    for (int q = 0; q < S.ns; ++q) words = std::max(words, (S.p[q].n + 31) / 32);
    if (g.wall) {
        k_implicit_push_tile<T, true><<<ntiles < cap ? ntiles : cap, kMoverThreads, smem, s>>>(g, t, mb, S, E, B, Et);
        k_implicit_push_deferred<T, true><<<grid_for(words, 128), 128, 0, s>>>(g, S, E, B, Et);
    } else {
        k_implicit_push_tile<T, false><<<ntiles < cap ? ntiles : cap, kMoverThreads, smem, s>>>(g, t, mb, S, E, B, Et);
        k_implicit_push_deferred<T, false><<<grid_for(words, 128), 128, 0, s>>>(g, S, E, B, Et);
    }
    return true;
}

template <typename T>
void PK<T>::implicit_push(cudaStream_t s, const GridP& g, PartView<T> p, double q, double m, const double* E,
                          const double* B, const double* Et) {
    if (p.n == 0) return;
    if (g.wall) k_implicit_push<T, true><<<grid_for(p.n, 128, 32), 128, 0, s>>>(g, p, q, m, E, B, Et);
    else k_implicit_push<T, false><<<grid_for(p.n, 128, 32), 128, 0, s>>>(g, p, q, m, E, B, Et);
}

template <typename T>
void PK<T>::density_deposit(cudaStream_t s, const GridP& g, PartView<T> p, double m, double w, double* conc,
                            double* energy, double* mom) {
    if (p.n == 0) return;
    k_density_deposit<T><<<grid_for(p.n, 256, 32), 256, 0, s>>>(g, p, m, w, conc, energy, mom);
}

template <typename T>
void PK<T>::gather_payload(cudaStream_t s, const int* perm, long long n, PartView<T> src, PartView<T> dst) {
    if (n == 0) return;
    k_gather_payload<T><<<grid_for(n, 256, 32), 256, 0, s>>>(perm, n, src, dst);
}

template <typename T>
void PK<T>::particle_sums(cudaStream_t s, PartView<T> p, double m, double w, double* partials, int P) {
    k_particle_sums<T><<<P, kRedThreads, 0, s>>>(p, m, w, partials, P);
}

template <typename T>
void PK<T>::field_sq_partials(cudaStream_t s, const void* F, long long n, double* partials, int P) {
    k_sq_partials<T><<<P, kRedThreads, 0, s>>>((const T*)F, n, partials);
}

template <typename T>
void PK<T>::to_real(cudaStream_t s, const double* src, void* dst, long long n) {
    if (n == 0) return;
    k_convert<T><<<grid_for(n, 256), 256, 0, s>>>(src, (T*)dst, n);
}

template <typename T>
void PK<T>::to_real_checked(cudaStream_t s, const double* src, void* dst, long long n, int mode, int* flag) {
    if (n == 0) return;
    k_convert_checked<T><<<grid_for(n, 256), 256, 0, s>>>(src, (T*)dst, n, mode, flag);
}

template <typename T>
void PK<T>::from_real(cudaStream_t s, const void* src, double* dst, long long n) {
    if (n == 0) return;
    k_convert_back<T><<<grid_for(n, 256), 256, 0, s>>>((const T*)src, dst, n);
}

}  // namespace pic
