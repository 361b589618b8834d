// kernels.hpp -- host-side launchers of the CUDA kernels, shared by the C ABI
// (api.cu).  Particle kernels exist for FP32 and FP64 particle state
// (kernels_f32.cu, kernels_f64.cu); grid and Krylov kernels are FP64 only
// (grid.cu).
#pragma once
#include <cuda_runtime.h>
#include <vector>
#include "common.cuh"
#include "types.cuh"

namespace pic {

constexpr int kNumSM = 152;

inline int grid_for(long long n, int threads, int per_sm = 16) {
    long long b = (n + threads - 1) / threads;
    long long cap = (long long)kNumSM * per_sm;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

// Number of partial sums used by every deterministic reduction of n items.
inline int red_blocks(long long n) {
    long long b = (n + 255) / 256;
    if (b > 1024) b = 1024;
    if (b < 1) b = 1;
    return (int)b;
}

template <typename T>
struct PK {
    // with GridP::wall the B half step first sets the ghost column left of
    // the wall, and the E step writes er[1], er[2] on the open boundary node
    static void yee_b_half(cudaStream_t s, const GridP& g, void* E, void* B);
    static void yee_e(cudaStream_t s, const GridP& g, void* E, const void* B, const double* J, const double er[3]);
    static void boris_push(cudaStream_t s, const GridP& g, PartView<T> p, double q, double m, const void* E,
                           const void* B);
    static void zigzag(cudaStream_t s, const GridP& g, PartView<T> p, double q, double m, double w, double* J);
    // fused gather/push/deposit over tiles (boris_tile.cuh); smem bytes and
    // grid size chosen by the caller
    static void push_deposit_tiled(cudaStream_t s, const GridP& g, const TileGeom& t, const TileShape& sh,
                                   const SpeciesSet<T>& S, const void* E, const void* B, double* Jpart, double* Jfix,
                                   int grid, size_t smem);
    // J from the tile partials and Jfix; inv_scale = 1 / fixed_scale for FP32
    // particles (integer partials), unused for FP64
    static void assemble_j(cudaStream_t s, const GridP& g, const TileGeom& t, const TileShape& sh, const double* Jpart,
                           const double* Jfix, double* J, double inv_scale);
    static float fixed_scale(const GridP& g, const SpeciesSet<T>& S);
    static size_t tile_smem_bytes(const TileShape& sh);
    static void implicit_deposit(cudaStream_t s, const GridP& g, PartView<T> p, double q, double m, double w,
                                 const double* E, const double* B, double* J, double* mu, double* rho, double* Pi,
                                 int compat, const GhostAxes& ga);
    // tiled deposit (implicit_tile.cuh), periodic pressure placement; needs
    // tile-major sorted particles
    static ImpBlock implicit_block(const GridP& g, const TileGeom& t, int h);
    static size_t implicit_tile_smem(const ImpBlock& bk);
    static void implicit_deposit_tiled(cudaStream_t s, const GridP& g, const TileGeom& t, const ImpBlock& bk,
                                       const ImpSpecies<T>& S, const T* E, const T* B, double* J,
                                       double* mu, double* rho, double* Pi);
    // tiled mover (implicit_tile.cuh): fields staged per tile; needs
    // tile-major sorted particles; false if the blocks do not fit
    static bool implicit_push_tiled(cudaStream_t s, const GridP& g, const TileGeom& t, const ImpSpecies<T>& S,
                                    const double* E, const double* B, const double* Et);
    static void implicit_push(cudaStream_t s, const GridP& g, PartView<T> p, double q, double m, const double* E,
                              const double* B, const double* Et);
    static void gather_payload(cudaStream_t s, const int* perm, long long n, PartView<T> src, PartView<T> dst);
    // updateDensityParameters deposit of one species (diag.cuh)
    static void density_deposit(cudaStream_t s, const GridP& g, PartView<T> p, double m, double w, double* conc,
                                double* energy, double* mom);
    static void particle_sums(cudaStream_t s, PartView<T> p, double m, double w, double* partials, int P);
    static void field_sq_partials(cudaStream_t s, const void* F, long long n, double* partials, int P);
    static void to_real(cudaStream_t s, const double* src, void* dst, long long n);
    static void to_real_checked(cudaStream_t s, const double* src, void* dst, long long n, int mode, int* flag);
    static void from_real(cudaStream_t s, const void* src, double* dst, long long n);
    static void validate(cudaStream_t s, const GridP& g, PartView<T> p, int* flag);
    static void iota(cudaStream_t s, int* a, long long n, long long start = 0);
};

// init.cu
std::vector<double> juttner_table(double theta, int n, std::vector<double>& us);
template <typename T>
void launch_fill(cudaStream_t s, PartView<T> p, long long ppc, unsigned long long seed, const double* u, const double* c,
                 int ntab, double mass, double drift_gamma, int alternate, int rowx, int nx, int x0);

// grid.cu
void launch_keys_hist(cudaStream_t s, const GridP& g, const TileGeom& t, const int* cell, long long n, int* key,
                      int* counts);
void launch_excl_scan(cudaStream_t s, int* a, long long n, int* block_sums, int* grand_total);
void launch_scatter_atomic(cudaStream_t s, const int* key, long long n, int* cursor, int* tmp);
void launch_segsort(cudaStream_t s, const int* off, int nkeys, const int* tmp, int* perm, int* long_count,
                    int* long_list);
void launch_pi_fold_reference(cudaStream_t s, double* P, const GhostAxes& ga, int axis);
void launch_jg_build(cudaStream_t s, const GridP& g, const GhostAxes& ga, const double* J, const double* P,
                     double* Jg, int nex, int ney, int nez);
void launch_rho_ext_reference(cudaStream_t s, const GridP& g, const double* Jg, int nex, int ney, int nez,
                              const double* rho, double* rho_ext, int ex, int ey, int ez);
void launch_jg_interior(cudaStream_t s, const GridP& g, const double* Jg, int nex, int ney, int nez, int gx, int gy,
                        int gz, double* J);
void launch_j_minus_divpi(cudaStream_t s, const GridP& g, const double* Pi, const double* Jin, double* Jout);
void launch_rho_ext_periodic(cudaStream_t s, const GridP& g, const double* J, const double* rho, double* rho_ext,
                             int ex, int ey, int ez);
void launch_maxwell_rhs(cudaStream_t s, const GridP& g, const double* E, const double* B, const double* J,
                        const double* rho_ext, int ex, int ey, double* rhs);
// y = A(mu) x; wmu: scratch of 3N doubles (mu x)
void launch_maxwell_apply(cudaStream_t s, const GridP& g, const OpCoef& oc, const double* mu, const double* x,
                          double* y, double* wmu);
void launch_maxwell_apply_f32(cudaStream_t s, const GridP& g, const OpCoef& oc, const float* mu, const float* x,
                              float* y, float* wmu, const unsigned* skip);
// conductor wall at x = 0 / open boundary at x = (nx - 2) dx (wall.cuh)
void launch_wall_moments(cudaStream_t s, const GridP& g, double* J, double* mu, double* rho, double* Pi,
                         int pi_mirror);
void launch_wall_zero_j(cudaStream_t s, const GridP& g, double* J);
void launch_wall_rhs(cudaStream_t s, const GridP& g, const double* rho_ext, int ex, int ey, const double er[3],
                     double* rhs);
void launch_wall_b(cudaStream_t s, const GridP& g, double* B, const double br[3]);
void launch_maxwell_apply_t(cudaStream_t s, const GridP& g, const OpCoef& oc, const double* mu, const double* y,
                            double* out);
void launch_field_update(cudaStream_t s, const GridP& g, const double* Et, const double* E, const double* B,
                         double* En, double* Bn, int doE, int doB);
void launch_smooth(cudaStream_t s, const GridP& g, const double* src, double* dst, int ncomp, double sp);
void launch_smooth_rho_ext(cudaStream_t s, const GridP& g, const double* src, double* dst, int ex, int ey, int ez,
                           double sp);
void launch_density_finish(cudaStream_t s, long long N, double q, const double* conc, const double* energy,
                           double* mom_to_vel, double* rho);
void launch_density_wall_fold(cudaStream_t s, const GridP& g, double* conc, double* energy, double* mom);
// Krylov
void launch_dot(cudaStream_t s, const double* a, const double* b, long long n, double* partials, int P, double* out,
                int take_sqrt);
void launch_multi_dot(cudaStream_t s, const double* V, long long ld, int k, const double* w, long long n,
                      double* partials, int P, double* out);
void launch_axpy_minus_dev(cudaStream_t s, double* y, const double* x, const double* alpha, long long n);
void launch_multi_axpy_minus(cudaStream_t s, double* w, const double* V, long long ld, int k, const double* h,
                             int hstride, long long n);
void launch_scale_inv_dev(cudaStream_t s, double* v, const double* w, const double* h, long long n);
void launch_scale(cudaStream_t s, double* v, const double* w, double sc, long long n);
void launch_div(cudaStream_t s, double* v, const double* w, double d, long long n);
void launch_combine(cudaStream_t s, double* x, const double* V, long long ld, int k, const double* y, double scale,
                    int accumulate, long long n);
// Offsets of the inner solve's FP64 scalars (one array): [0] |v|^2, [1]
// |v|, then the Hessenberg columns (column j at h + j (S + 1), rows 0..j),
// the squared norms of the new basis vectors, the least-squares solution y,
// the Givens cosines and sines and the rotated right part g.
struct InnerLayout {
    int S;
    __host__ __device__ long long h() const { return 8; }
    __host__ __device__ long long hn() const { return 8 + (long long)(S + 1) * S; }
    __host__ __device__ long long y() const { return hn() + S; }
    __host__ __device__ long long cs() const { return y() + S + 1; }
    __host__ __device__ long long sn() const { return cs() + S; }
    __host__ __device__ long long g() const { return sn() + S; }
    __host__ __device__ long long size() const { return g() + S + 1; }
};

// FP32 vectors of the mixed-precision preconditioner (FP64 partials, outputs
// and coefficients; each reduction one launch, finished by its last block,
// counter: a zeroed device word; skip: the inner solve's done flag, the
// kernel returns at once when it is set)
void launch_dot_f32(cudaStream_t s, const float* a, const float* b, long long n, double* partials, int P,
                    double* out, unsigned* counter);
void launch_multi_dot_f32(cudaStream_t s, const float* V, long long ld, int k, const float* w, long long n,
                          double* partials, int P, double* out, unsigned* counter, const unsigned* skip);
void launch_axpy_norm_f32(cudaStream_t s, float* w, const float* V, long long ld, int k, const double* h, long long n,
                          double* partials, int P, double* out, unsigned* counter, const unsigned* skip);
void launch_normalize_f32(cudaStream_t s, float* v, const float* w, const double* h2, long long n,
                          const unsigned* skip);
void launch_to_f32(cudaStream_t s, float* dst, const double* src, long long n);
void launch_combine_f32(cudaStream_t s, double* z, const float* V, long long ld, const unsigned* kp, const double* y,
                        double scale, long long n);
// Givens step j and back-substitution of the inner least-squares problem
// (scalars laid out as InnerLayout{S} in h; flags: [1] done, [2] columns)
void launch_inner_givens(cudaStream_t s, int j, int S, double* h, double tol, unsigned* flags);
void launch_inner_backsolve(cudaStream_t s, int S, double* h, unsigned* flags);
void launch_residual(cudaStream_t s, double* r, const double* b, const double* Ax, long long n);
void launch_nonfinite(cudaStream_t s, const double* a, long long n, int* flag);
void launch_finalize(cudaStream_t s, const double* partials, int P, int nvec, double* out, int ostride, int take_sqrt);

}  // namespace pic
