// grid.cu -- launchers of the FP64 grid kernels: cell sort, implicit moment
// corrections, Maxwell right part and operator, field update, Krylov vectors.
#include "implicit_grid.cuh"
#include "kernels.hpp"
#include "krylov.cuh"
#include "sort.cuh"
#include "wall.cuh"
#include <algorithm>
#include <cstdint>
#include <initializer_list>

namespace pic {

// ---------------------------------------------------------------- sort
void launch_keys_hist(cudaStream_t s, const GridP& g, const TileGeom& t, const int* cell, long long n, int* key,
                      int* counts) {
    if (n == 0) return;
    k_keys_hist<<<grid_for(n, 256, 32), 256, 0, s>>>(g, t, cell, n, key, counts);
}

void launch_excl_scan(cudaStream_t s, int* a, long long n, int* block_sums, int* grand_total) {
    const long long per = (long long)kScanThreads * kScanItems;
    const int nb = (int)((n + per - 1) / per);
    k_scan_blocks<<<nb, kScanThreads, 0, s>>>(a, n, block_sums);
    k_scan_top<<<1, kScanThreads, 0, s>>>(block_sums, nb, grand_total);
    k_scan_add<<<nb, kScanThreads, 0, s>>>(a, n, block_sums);
}

void launch_scatter_atomic(cudaStream_t s, const int* key, long long n, int* cursor, int* tmp) {
    if (n == 0) return;
    k_scatter_atomic<<<grid_for(n, 256, 32), 256, 0, s>>>(key, n, cursor, tmp);
}

void launch_segsort(cudaStream_t s, const int* off, int nkeys, const int* tmp, int* perm, int* long_count,
                    int* long_list) {
    cudaMemsetAsync(long_count, 0, sizeof(int), s);
    long long warps = nkeys;
    int blocks = (int)std::min<long long>((warps * 32 + 255) / 256, (long long)kNumSM * 32);
    k_segsort_warp<<<blocks, 256, 0, s>>>(off, nkeys, tmp, perm, long_count, long_list);
    k_segsort_block<<<kNumSM, 1024, 0, s>>>(off, long_list, long_count, tmp, perm);
}

// ---------------------------------------------------------------- moments
void launch_pi_fold_reference(cudaStream_t s, double* P, const GhostAxes& ga, int axis) {
    const int ce[3] = {ga.cex, ga.cey, ga.cez};
    if (ce[axis] == 1) return;   // single-cell axis: nothing to fold
    const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
    long long total = 9LL * ce[a1] * ce[a2];
    k_pi_fold_reference<<<grid_for(total, 256), 256, 0, s>>>(P, ga, axis);
}

void launch_jg_build(cudaStream_t s, const GridP& g, const GhostAxes& ga, const double* J, const double* P,
                     double* Jg, int nex, int ney, int nez) {
    long long n = (long long)nex * ney * nez;
    k_jg_build<<<grid_for(n, 256), 256, 0, s>>>(g, ga, J, P, Jg, nex, ney, nez);
}

void launch_rho_ext_reference(cudaStream_t s, const GridP& g, const double* Jg, int nex, int ney, int nez,
                              const double* rho, double* rho_ext, int ex, int ey, int ez) {
    long long n = (long long)ex * ey * ez;
    k_rho_ext_reference<<<grid_for(n, 256), 256, 0, s>>>(g, Jg, nex, ney, nez, rho, rho_ext, ex, ey, ez);
}

void launch_jg_interior(cudaStream_t s, const GridP& g, const double* Jg, int nex, int ney, int nez, int gx, int gy,
                        int gz, double* J) {
    k_jg_interior<<<grid_for(g.N, 256), 256, 0, s>>>(g, Jg, nex, ney, nez, gx, gy, gz, J);
}

void launch_j_minus_divpi(cudaStream_t s, const GridP& g, const double* Pi, const double* Jin, double* Jout) {
    k_j_minus_divpi<<<grid_for(g.N, 256), 256, 0, s>>>(g, Pi, Jin, Jout);
}

void launch_rho_ext_periodic(cudaStream_t s, const GridP& g, const double* J, const double* rho, double* rho_ext,
                             int ex, int ey, int ez) {
    long long n = (long long)ex * ey * ez;
    k_rho_ext_periodic<<<grid_for(n, 256), 256, 0, s>>>(g, J, rho, rho_ext, ex, ey, ez);
}

void launch_maxwell_rhs(cudaStream_t s, const GridP& g, const double* E, const double* B, const double* J,
                        const double* rho_ext, int ex, int ey, double* rhs) {
    k_maxwell_rhs<<<grid_for(g.N, 256), 256, 0, s>>>(g, E, B, J, rho_ext, ex, ey, rhs);
}

void launch_maxwell_apply(cudaStream_t s, const GridP& g, const OpCoef& oc, const double* mu, const double* x,
                          double* y, double* wmu) {
    k_mu_times<double><<<grid_for(g.N, 256), 256, 0, s>>>(g.N, mu, x, wmu, nullptr);
    k_maxwell_stencil<double><<<grid_for(g.N, 256), 256, 0, s>>>(g, oc, x, wmu, y, nullptr);
    if (g.wall) k_wall_rows<double><<<grid_for((long long)g.ny * g.nz, 256), 256, 0, s>>>(g, x, y, nullptr);
}

// The same operator in FP32 (inner solve of the mixed-precision
// preconditioner; mu an FP32 copy).
void launch_maxwell_apply_f32(cudaStream_t s, const GridP& g, const OpCoef& oc, const float* mu, const float* x,
                              float* y, float* wmu, const unsigned* skip) {
    k_mu_times<float><<<grid_for(g.N, 256), 256, 0, s>>>(g.N, mu, x, wmu, skip);
    if (g.nx % ZM_TX == 0 && g.ny % ZM_TY == 0 && g.nz >= 3 && oc.has[0] && oc.has[1] && oc.has[2]) {
        const dim3 grid(g.nx / ZM_TX, g.ny / ZM_TY, (g.nz + ZM_ZC - 1) / ZM_ZC);
        k_maxwell_stencil_zm<<<grid, ZM_TX * ZM_TY, 0, s>>>(g, oc, x, wmu, y, skip);
    } else {
        k_maxwell_stencil<float><<<grid_for(g.N, 256), 256, 0, s>>>(g, oc, x, wmu, y, skip);
    }
    if (g.wall) k_wall_rows<float><<<grid_for((long long)g.ny * g.nz, 256), 256, 0, s>>>(g, x, y, skip);
}

void launch_wall_moments(cudaStream_t s, const GridP& g, double* J, double* mu, double* rho, double* Pi,
                         int pi_mirror) {
    k_wall_moments<<<grid_for((long long)g.ny * g.nz, 256), 256, 0, s>>>(g, J, mu, rho, Pi, pi_mirror);
}

void launch_wall_zero_j(cudaStream_t s, const GridP& g, double* J) {
    k_wall_zero_j<<<grid_for((long long)g.ny * g.nz, 256), 256, 0, s>>>(g, J);
}

void launch_wall_rhs(cudaStream_t s, const GridP& g, const double* rho_ext, int ex, int ey, const double er[3],
                     double* rhs) {
    k_wall_rhs<<<grid_for((long long)g.ny * g.nz, 256), 256, 0, s>>>(g, rho_ext, ex, ey, er[0], er[1], er[2], rhs);
}

void launch_wall_b(cudaStream_t s, const GridP& g, double* B, const double br[3]) {
    k_wall_b<<<grid_for((long long)g.ny * g.nz, 256), 256, 0, s>>>(g, B, br[0], br[1], br[2]);
}

void launch_maxwell_apply_t(cudaStream_t s, const GridP& g, const OpCoef& oc, const double* mu, const double* y,
                            double* out) {
    k_maxwell_apply_t<<<grid_for(g.N, 256), 256, 0, s>>>(g, oc, mu, y, out);
}

// One pass of the periodic 3x3x3 smoothing (createSmoothingMatrix and the
// smooth*Parameter loops, smoothing.cpp:105-137, 251-412, 535-739): weights
// s/2, 1-s, s/2 on every active axis, ncomp planar components, src -> dst.
__global__ void k_smooth27(GridP g, const double* __restrict__ src, double* __restrict__ dst, int ncomp, double sp) {
    const long long N = g.N;
    const double wside = sp / 2, wmid = 1.0 - sp;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N * ncomp;
         e += (long long)gridDim.x * blockDim.x) {
        const long long c = e / N, id = e - c * N;
        int i, j, k;
        decode(g, (int)id, i, j, k);
        const double* a = src + c * N;
        double s = 0.0;
        for (int dk = -1; dk <= 1; ++dk) {
            if (!g.z3 && dk) continue;
            const double wk = g.z3 ? (dk ? wside : wmid) : 1.0;
            for (int dj = -1; dj <= 1; ++dj) {
                if (!g.y3 && dj) continue;
                const double wj = g.y3 ? (dj ? wside : wmid) : 1.0;
                for (int di = -1; di <= 1; ++di) {
                    if (g.nx == 1 && di) continue;
                    const double wi = g.nx > 1 ? (di ? wside : wmid) : 1.0;
                    s += a[linw(g, i + di, j + dj, k + dk)] * (wi * wj * wk);
                }
            }
        }
        dst[e] = s;
    }
}

// The same pass on rho-hat stored with one low ghost layer (extent n + 1 on
// active axes, ext index e holds cell e - 1, so ext 0 is the periodic image
// of cell n - 1): every ext entry gets the smoothed value of its cell.
__global__ void k_smooth_rho_ext(GridP g, const double* __restrict__ src, double* __restrict__ dst, int ex, int ey,
                                 int ez, double sp) {
    const long long tot = (long long)ex * ey * ez;
    const double wside = sp / 2, wmid = 1.0 - sp;
    auto at = [&](int i, int j, int k) -> double {   // cell (i, j, k), periodic, from the ext array
        const int ri = g.nx > 1 ? wrap_any(i, g.nx) + 1 : 0;
        const int rj = g.y3 ? wrap_any(j, g.ny) + 1 : 0;
        const int rk = g.z3 ? wrap_any(k, g.nz) + 1 : 0;
        return src[((long long)rk * ey + rj) * ex + ri];
    };
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
        const int ri = (int)(e % ex), rj = (int)((e / ex) % ey), rk = (int)(e / ((long long)ex * ey));
        const int i = g.nx > 1 ? ri - 1 : 0, j = g.y3 ? rj - 1 : 0, k = g.z3 ? rk - 1 : 0;
        double s = 0.0;
        for (int dk = -1; dk <= 1; ++dk) {
            if (!g.z3 && dk) continue;
            const double wk = g.z3 ? (dk ? wside : wmid) : 1.0;
            for (int dj = -1; dj <= 1; ++dj) {
                if (!g.y3 && dj) continue;
                const double wj = g.y3 ? (dj ? wside : wmid) : 1.0;
                for (int di = -1; di <= 1; ++di) {
                    if (g.nx == 1 && di) continue;
                    const double wi = g.nx > 1 ? (di ? wside : wmid) : 1.0;
                    s += at(i + di, j + dj, k + dk) * (wi * wj * wk);
                }
            }
        }
        dst[e] = s;
    }
}

void launch_smooth(cudaStream_t s, const GridP& g, const double* src, double* dst, int ncomp, double sp) {
    k_smooth27<<<grid_for(g.N * ncomp, 256), 256, 0, s>>>(g, src, dst, ncomp, sp);
}

void launch_smooth_rho_ext(cudaStream_t s, const GridP& g, const double* src, double* dst, int ex, int ey, int ez,
                           double sp) {
    k_smooth_rho_ext<<<grid_for((long long)ex * ey * ez, 256), 256, 0, s>>>(g, src, dst, ex, ey, ez, sp);
}

// Bulk velocity = momentum density / energy density (0 where the energy
// density is 0), rho += q conc (momentum_collecting.cpp:960-1005).
__global__ void k_density_finish(long long N, double q, const double* __restrict__ conc,
                                 const double* __restrict__ energy, double* __restrict__ v, double* __restrict__ rho) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        const double e = energy[c];
        for (int d = 0; d < 3; ++d) v[d * N + c] = e > 0 ? v[d * N + c] / e : 0.0;
        rho[c] += q * conc[c];
    }
}

void launch_density_finish(cudaStream_t s, long long N, double q, const double* conc, const double* energy,
                           double* mom_to_vel, double* rho) {
    k_density_finish<<<grid_for(N, 256), 256, 0, s>>>(N, q, conc, energy, mom_to_vel, rho);
}

// Wall box (SUPER_CONDUCTOR_LEFT, one rank): the deposits in the ghost cell
// left of the wall (storage column nx - 1) go to cell 0 with the momentum's
// x component reflected (momentum_collecting.cpp:945-960); those beyond the
// open boundary (column nx - 2) go to the last physical cell nx - 3
// (sumCellParametersX, momentum_exchange.cpp:968-988, and
// sumCellVectorParametersX, 1351-1361); both ghost columns end empty.  One
// thread per (y, z) row: each touches four cells of its own row.
__global__ void k_density_wall_fold(GridP g, double* __restrict__ conc, double* __restrict__ energy,
                                    double* __restrict__ mom) {
    const int rows = g.ny * g.nz;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        const int j = r % g.ny, k = r / g.ny;
        const long long gl = lin(g, g.nx - 1, j, k), f = lin(g, 0, j, k);
        const long long gr = lin(g, g.nx - 2, j, k), l = lin(g, g.nx - 3, j, k);
        conc[f] += conc[gl];
        energy[f] += energy[gl];
        conc[l] += conc[gr];
        energy[l] += energy[gr];
        conc[gl] = energy[gl] = conc[gr] = energy[gr] = 0.0;
        for (int d = 0; d < 3; ++d) {
            double* m = mom + d * g.N;
            m[f] += d == 0 ? -m[gl] : m[gl];
            m[l] += m[gr];
            m[gl] = m[gr] = 0.0;
        }
    }
}

void launch_density_wall_fold(cudaStream_t s, const GridP& g, double* conc, double* energy, double* mom) {
    k_density_wall_fold<<<grid_for((long long)g.ny * g.nz, 128), 128, 0, s>>>(g, conc, energy, mom);
}

void launch_field_update(cudaStream_t s, const GridP& g, const double* Et, const double* E, const double* B,
                         double* En, double* Bn, int doE, int doB) {
    k_field_update<<<grid_for(g.N, 256), 256, 0, s>>>(g, Et, E, B, En, Bn, doE, doB);
}

// ---------------------------------------------------------------- Krylov
void launch_finalize(cudaStream_t s, const double* partials, int P, int nvec, double* out, int ostride,
                     int take_sqrt) {
    k_finalize<<<nvec, kRedThreads, 0, s>>>(partials, P, out, ostride, take_sqrt);
}

void launch_dot(cudaStream_t s, const double* a, const double* b, long long n, double* partials, int P, double* out,
                int take_sqrt) {
    k_dot_partials<<<P, kRedThreads, 0, s>>>(a, b, n, partials);
    k_finalize<<<1, kRedThreads, 0, s>>>(partials, P, out, 1, take_sqrt);
}

void launch_multi_dot(cudaStream_t s, const double* V, long long ld, int k, const double* w, long long n,
                      double* partials, int P, double* out) {
    for (int k0 = 0; k0 < k; k0 += 8)
        k_multi_dot_partials<8><<<P, kRedThreads, 0, s>>>(V, ld, k0, k, w, n, partials, P);
    k_finalize<<<k, kRedThreads, 0, s>>>(partials, P, out, 1, 0);
}

void launch_axpy_minus_dev(cudaStream_t s, double* y, const double* x, const double* alpha, long long n) {
    k_axpy_minus_dev<<<grid_for(n, 256), 256, 0, s>>>(y, x, alpha, n);
}

void launch_multi_axpy_minus(cudaStream_t s, double* w, const double* V, long long ld, int k, const double* h,
                             int hstride, long long n) {
    k_multi_axpy_minus<<<grid_for(n, 256), 256, 0, s>>>(w, V, ld, k, h, hstride, n);
}

void launch_scale_inv_dev(cudaStream_t s, double* v, const double* w, const double* h, long long n) {
    k_scale_inv_dev<<<grid_for(n, 256), 256, 0, s>>>(v, w, h, n);
}

void launch_scale(cudaStream_t s, double* v, const double* w, double sc, long long n) {
    k_scale<<<grid_for(n, 256), 256, 0, s>>>(v, w, sc, n);
}

void launch_div(cudaStream_t s, double* v, const double* w, double d, long long n) {
    k_div<<<grid_for(n, 256), 256, 0, s>>>(v, w, d, n);
}

void launch_combine(cudaStream_t s, double* x, const double* V, long long ld, int k, const double* y, double scale,
                    int accumulate, long long n) {
    k_combine<<<grid_for(n, 256), 256, 0, s>>>(x, V, ld, k, y, scale, accumulate, n);
}

void launch_residual(cudaStream_t s, double* r, const double* b, const double* Ax, long long n) {
    k_residual<<<grid_for(n, 256), 256, 0, s>>>(r, b, Ax, n);
}

// FP32 vectors: float4 accesses when the length is a multiple of 4 and the
// bases are 16-byte aligned.
static bool vec4_ok(long long n, std::initializer_list<const void*> ps) {
    if (n % 4) return false;
    for (const void* p : ps)
        if (reinterpret_cast<uintptr_t>(p) % 16) return false;
    return true;
}

void launch_dot_f32(cudaStream_t s, const float* a, const float* b, long long n, double* partials, int P,
                    double* out, unsigned* counter) {
    if (vec4_ok(n, {a, b})) k_dot_f32<4><<<P, kRedThreads, 0, s>>>(a, b, n / 4, partials, out, counter);
    else k_dot_f32<1><<<P, kRedThreads, 0, s>>>(a, b, n, partials, out, counter);
}

void launch_multi_dot_f32(cudaStream_t s, const float* V, long long ld, int k, const float* w, long long n,
                          double* partials, int P, double* out, unsigned* counter, const unsigned* skip) {
    const bool v4 = vec4_ok(n, {V, w}) && ld % 4 == 0;
    for (int k0 = 0; k0 < k; k0 += 8) {
        if (v4)
            k_multi_dot_f32<8, 4><<<P, kRedThreads, 0, s>>>(V, ld / 4, k0, k, w, n / 4, partials, out, counter, skip);
        else
            k_multi_dot_f32<8, 1><<<P, kRedThreads, 0, s>>>(V, ld, k0, k, w, n, partials, out, counter, skip);
    }
}

void launch_axpy_norm_f32(cudaStream_t s, float* w, const float* V, long long ld, int k, const double* h, long long n,
                          double* partials, int P, double* out, unsigned* counter, const unsigned* skip) {
    if (vec4_ok(n, {V, w}) && ld % 4 == 0)
        k_axpy_norm_f32<4><<<P, kRedThreads, 0, s>>>(w, V, ld / 4, k, h, n / 4, partials, out, counter, skip);
    else
        k_axpy_norm_f32<1><<<P, kRedThreads, 0, s>>>(w, V, ld, k, h, n, partials, out, counter, skip);
}

void launch_normalize_f32(cudaStream_t s, float* v, const float* w, const double* h2, long long n,
                          const unsigned* skip) {
    if (vec4_ok(n, {v, w})) k_normalize_f32<4><<<grid_for(n / 4, 256), 256, 0, s>>>(v, w, h2, n / 4, skip);
    else k_normalize_f32<1><<<grid_for(n, 256), 256, 0, s>>>(v, w, h2, n, skip);
}

void launch_inner_givens(cudaStream_t s, int j, int S, double* h, double tol, unsigned* flags) {
    k_inner_givens<<<1, 32, 0, s>>>(j, InnerLayout{S}, h, tol, flags);
}

void launch_inner_backsolve(cudaStream_t s, int S, double* h, unsigned* flags) {
    k_inner_backsolve<<<1, 32, 0, s>>>(InnerLayout{S}, h, flags);
}

void launch_to_f32(cudaStream_t s, float* dst, const double* src, long long n) {
    k_to_f32<<<grid_for(n, 256), 256, 0, s>>>(dst, src, n);
}

void launch_combine_f32(cudaStream_t s, double* z, const float* V, long long ld, const unsigned* kp, const double* y,
                        double scale, long long n) {
    k_combine_f32<<<grid_for(n, 256), 256, 0, s>>>(z, V, ld, kp, y, scale, n);
}

void launch_nonfinite(cudaStream_t s, const double* a, long long n, int* flag) {
    k_nonfinite<<<grid_for(n, 256), 256, 0, s>>>(a, n, flag);
}

}  // namespace pic
