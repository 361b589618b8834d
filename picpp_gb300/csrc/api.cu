// api.cu -- the C ABI (include/picpp_gb300.h): one context per simulation,
// owning every device buffer, one CUDA stream, status codes instead of exit().
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/picpp_gb300.h"
#include "kernels.hpp"
#include "nn.hpp"
#include "solver.hpp"

using namespace pic;

namespace {

struct Species {
    double q = 0, m = 1, w = 1;
    long long n = 0, cap = 0;
    int* cell = nullptr;
    int* id = nullptr;
    void* a[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};   // ox oy oz px py pz
    int* cell2 = nullptr;
    int* id2 = nullptr;
    void* b[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int* perm = nullptr;
    int* off = nullptr;     // nkeys + 1
    unsigned* defer = nullptr;   // 2 * dwords: the fused explicit kernel's push-later and deposit-later bits
    long long dwords = 0;
    bool sorted = false;
    long long next_id = 0;  // id of the next appended particle when the caller gives none
};

template <typename T>
PartView<T> view(Species& s) {
    return PartView<T>{s.cell, (T*)s.a[0], (T*)s.a[1], (T*)s.a[2], (T*)s.a[3], (T*)s.a[4], (T*)s.a[5], s.id, s.n};
}
template <typename T>
PartView<T> view_alt(Species& s) {
    return PartView<T>{s.cell2, (T*)s.b[0], (T*)s.b[1], (T*)s.b[2], (T*)s.b[3], (T*)s.b[4], (T*)s.b[5], s.id2, s.n};
}

}  // namespace

struct pic_ctx {
    pic_config cfg{};
    GridP g{};
    TileGeom tg{};
    TileShape ts{};
    GhostAxes ga{};
    int nkeys = 0, ntiles = 0, T3 = 0;
    int preal = 0;
    size_t rsz = 4;
    cudaStream_t s = nullptr;
    std::string err;
    std::vector<Species> sp;
    long long step = 0;
    // explicit (Yee) grids in particle precision, current in FP64
    void* E = nullptr;
    void* B = nullptr;
    double* J = nullptr;
    double* Jfix = nullptr;
    void* Jpart = nullptr;
    // implicit grids (FP64)
    double *Ei = nullptr, *Bi = nullptr, *Jh = nullptr, *mu = nullptr, *rho = nullptr, *rho_ext = nullptr;
    double *Pi = nullptr, *Jg = nullptr, *rhs = nullptr, *Et = nullptr, *En = nullptr, *Bn = nullptr;
    long long pi_len = 0, jg_len = 0, rho_ext_len = 0;
    int nex = 1, ney = 1, nez = 1, ex = 1, ey = 1, ez = 1;
    bool moments_ready = false, efield_ready = false;
    bool mu_valid = false;   // ctx->mu holds an operator (moments or an uploaded mu)
    Net* net = nullptr;      // learned preconditioner, created by pic_nn_init / pic_nn_set_params
    TripleStore trip;        // recorded (b, mu, x) triples of plain solves (pic_nn_record)
    double* smooth_tmp = nullptr;   // scratch of the smoothing passes (max(9N, rho-hat ext))
    bool fresh_sort = false;        // particles sorted and not moved since
    bool pending_compact = false;   // escaped particles (cell -1) not yet erased (wall boxes)
    double e_right[3] = {0, 0, 0}, b_right[3] = {0, 0, 0};   // open boundary fields (wall boxes)
    float* fields32 = nullptr;      // FP32 copies of E^n, B^n (6N) for the FP32 deposit
    // updateDensityParameters grids: per species conc, energy, velocity (5N), charge density (N)
    double* dens = nullptr;
    double* dens_rho = nullptr;
    int dens_ns = 0;
    // sort scratch
    int *key = nullptr, *counts = nullptr, *cursor = nullptr, *tmp = nullptr, *block_sums = nullptr;
    int *long_count = nullptr, *long_list = nullptr;
    long long sort_cap = 0;
    // staging and reductions
    double* stage = nullptr;
    long long stage_len = 0;
    double* partials = nullptr;
    int* flag = nullptr;
    Krylov kry;
    // phase timing (pic_profile)
    bool prof_on = false;
    struct Mark { int phase; cudaEvent_t a, b; };
    std::vector<Mark> marks;
    double prof_ms[PIC_PHASE_COUNT] = {};
    long launches = 0;
};

namespace {

// Folds recorded event pairs into the per-phase totals.
void prof_fold(pic_ctx* c) {
    if (c->marks.empty()) return;
    cudaStreamSynchronize(c->s);
    for (auto& m : c->marks) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, m.a, m.b) == cudaSuccess) c->prof_ms[m.phase] += ms;
        cudaEventDestroy(m.a);
        cudaEventDestroy(m.b);
    }
    c->marks.clear();
}

// Brackets one phase with CUDA events on the context stream while profiling.
struct Phase {
    pic_ctx* c;
    int ph;
    cudaEvent_t a = nullptr;
    Phase(pic_ctx* ctx, int phase, int nkernels) : c(ctx), ph(phase) {
        if (!c->prof_on) return;
        c->launches += nkernels;
        cudaEventCreate(&a);
        cudaEventRecord(a, c->s);
    }
    ~Phase() {
        if (!c->prof_on || !a) return;
        cudaEvent_t b;
        cudaEventCreate(&b);
        cudaEventRecord(b, c->s);
        c->marks.push_back({ph, a, b});
        if (c->marks.size() > 2048) prof_fold(c);
    }
};

}  // namespace

namespace {

pic_status fail(pic_ctx* c, pic_status st, const std::string& m) {
    if (c) c->err = m;
    return st;
}

pic_status cuda_fail(pic_ctx* c, cudaError_t e, const char* where) {
    return fail(c, PIC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(expr)                                                   \
    do {                                                           \
        cudaError_t e_ = (expr);                                   \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #expr);   \
    } while (0)

#define CKL(ctx, where)                                            \
    do {                                                           \
        cudaError_t e_ = cudaGetLastError();                       \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, where);   \
    } while (0)

template <typename P>
cudaError_t dalloc(P** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    return cudaMalloc((void**)p, bytes);
}

pic_status sync(pic_ctx* ctx, const char* where) {
    cudaError_t e = cudaStreamSynchronize(ctx->s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, where);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, where);
    return PIC_OK;
}

bool is_buneman(const pic_ctx* c) { return c->cfg.solver == PIC_SOLVER_BUNEMAN; }

// -------------------------------------------------------------- sort
template <typename T>
pic_status sort_species(pic_ctx* ctx, Species& sp) {
    Phase ph(ctx, PIC_PHASE_SORT, 8);
    cudaStream_t s = ctx->s;
    const long long n = sp.n;
    CK(cudaMemsetAsync(ctx->counts, 0, sizeof(int) * ((size_t)ctx->nkeys + 1), s));
    launch_keys_hist(s, ctx->g, ctx->tg, sp.cell, n, ctx->key, ctx->counts);
    launch_excl_scan(s, ctx->counts, (long long)ctx->nkeys + 1, ctx->block_sums, nullptr);
    CK(cudaMemcpyAsync(sp.off, ctx->counts, sizeof(int) * ((size_t)ctx->nkeys + 1), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(ctx->cursor, ctx->counts, sizeof(int) * (size_t)ctx->nkeys, cudaMemcpyDeviceToDevice, s));
    launch_scatter_atomic(s, ctx->key, n, ctx->cursor, ctx->tmp);
    launch_segsort(s, sp.off, ctx->nkeys, ctx->tmp, sp.perm, ctx->long_count, ctx->long_list);
    long long kept = n;
    if (ctx->g.wall) {
        // particles that escaped (cell -1) have no key: the keyed ones, in
        // key order, are the species from now on (eraseEscapedPaticles,
        // mover.cpp:167-192)
        int total = 0;
        CK(cudaMemcpyAsync(&total, sp.off + ctx->nkeys, sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        kept = total;
    }
    PK<T>::gather_payload(s, sp.perm, kept, view<T>(sp), view_alt<T>(sp));
    CKL(ctx, "sort");
    std::swap(sp.cell, sp.cell2);
    std::swap(sp.id, sp.id2);
    for (int q = 0; q < 6; ++q) std::swap(sp.a[q], sp.b[q]);
    sp.n = kept;
    sp.sorted = true;
    return PIC_OK;
}

pic_status sort_all(pic_ctx* ctx) {
    for (auto& sp : ctx->sp) {
        pic_status st = ctx->preal ? sort_species<double>(ctx, sp) : sort_species<float>(ctx, sp);
        if (st != PIC_OK) return st;
    }
    ctx->fresh_sort = true;
    ctx->pending_compact = false;
    return PIC_OK;
}

// Erases the particles that left a wall box since the last sort, before any
// call that reads the particle arrays.
pic_status settle(pic_ctx* ctx) {
    if (!ctx->pending_compact) return PIC_OK;
    return sort_all(ctx);
}

bool all_sorted(const pic_ctx* ctx) {
    for (const auto& sp : ctx->sp)
        if (!sp.sorted) return false;
    return true;
}

pic_status ensure_smooth_tmp(pic_ctx* ctx) {
    if (ctx->smooth_tmp) return PIC_OK;
    const size_t n = std::max<size_t>(9 * (size_t)ctx->g.N, (size_t)ctx->rho_ext_len);
    CK(dalloc(&ctx->smooth_tmp, sizeof(double) * n));
    return PIC_OK;
}

// smoothingCount passes over the explicit current (simulation.cpp:186-188).
pic_status smooth_current(pic_ctx* ctx) {
    if (ctx->cfg.smoothing_count <= 0) return PIC_OK;
    pic_status st = ensure_smooth_tmp(ctx);
    if (st != PIC_OK) return st;
    const size_t L = 3 * (size_t)ctx->g.N;
    for (int q = 0; q < ctx->cfg.smoothing_count; ++q) {
        launch_smooth(ctx->s, ctx->g, ctx->J, ctx->smooth_tmp, 3, ctx->cfg.smoothing_parameter);
        CK(cudaMemcpyAsync(ctx->J, ctx->smooth_tmp, sizeof(double) * L, cudaMemcpyDeviceToDevice, ctx->s));
    }
    return PIC_OK;
}

// smoothingCount passes over rho-hat, J-hat and mu (simulation.cpp:213-217).
pic_status smooth_moments(pic_ctx* ctx) {
    if (ctx->cfg.smoothing_count <= 0) return PIC_OK;
    pic_status st = ensure_smooth_tmp(ctx);
    if (st != PIC_OK) return st;
    const GridP& g = ctx->g;
    const double sp = ctx->cfg.smoothing_parameter;
    cudaStream_t s = ctx->s;
    for (int q = 0; q < ctx->cfg.smoothing_count; ++q) {
        launch_smooth_rho_ext(s, g, ctx->rho_ext, ctx->smooth_tmp, ctx->ex, ctx->ey, ctx->ez, sp);
        CK(cudaMemcpyAsync(ctx->rho_ext, ctx->smooth_tmp, sizeof(double) * ctx->rho_ext_len, cudaMemcpyDeviceToDevice, s));
        launch_smooth(s, g, ctx->Jh, ctx->smooth_tmp, 3, sp);
        CK(cudaMemcpyAsync(ctx->Jh, ctx->smooth_tmp, sizeof(double) * 3 * g.N, cudaMemcpyDeviceToDevice, s));
        launch_smooth(s, g, ctx->mu, ctx->smooth_tmp, 9, sp);
        CK(cudaMemcpyAsync(ctx->mu, ctx->smooth_tmp, sizeof(double) * 9 * g.N, cudaMemcpyDeviceToDevice, s));
    }
    return PIC_OK;
}

// -------------------------------------------------------------- explicit
template <typename T>
pic_status buneman_steps(pic_ctx* ctx, int nsteps) {
    cudaStream_t s = ctx->s;
    const GridP& g = ctx->g;
    for (int it = 0; it < nsteps; ++it) {
        if (ctx->cfg.sort_every > 0 && (!all_sorted(ctx) || ctx->step % ctx->cfg.sort_every == 0)) {
            pic_status st = sort_all(ctx);
            if (st != PIC_OK) return st;
        }
        {
            Phase ph(ctx, PIC_PHASE_FIELDS, 1);
            PK<T>::yee_b_half(s, g, ctx->E, ctx->B);
            CK(cudaMemsetAsync(ctx->Jfix, 0, sizeof(double) * 3 * g.N, s));
        }
        if (all_sorted(ctx)) {
            SpeciesSet<T> S{};
            S.ns = (int)ctx->sp.size();
            for (int q = 0; q < S.ns; ++q) {
                S.p[q] = view<T>(ctx->sp[q]);
                S.q[q] = T(ctx->sp[q].q); S.m[q] = T(ctx->sp[q].m); S.w[q] = T(ctx->sp[q].w);
                S.off[q] = ctx->sp[q].off;
                S.defer[q] = ctx->sp[q].defer;
                S.dwords[q] = ctx->sp[q].dwords;
            }
            int grid = ctx->ntiles < kNumSM * 8 ? ctx->ntiles : kNumSM * 8;
            {
                Phase ph(ctx, PIC_PHASE_PUSH_DEPOSIT, 2);   // the fused kernel and its deferred pass
                PK<T>::push_deposit_tiled(s, g, ctx->tg, ctx->ts, S, ctx->E, ctx->B, (double*)ctx->Jpart, ctx->Jfix,
                                          grid, PK<T>::tile_smem_bytes(ctx->ts));
            }
            {
                Phase ph(ctx, PIC_PHASE_FIELDS, 1);
                PK<T>::yee_b_half(s, g, ctx->E, ctx->B);
            }
            {
                Phase ph(ctx, PIC_PHASE_ASSEMBLE, 1);
                PK<T>::assemble_j(s, g, ctx->tg, ctx->ts, (const double*)ctx->Jpart, ctx->Jfix, ctx->J,
                                  1.0 / (double)PK<T>::fixed_scale(g, S));
            }
        } else {
            {
                Phase ph(ctx, PIC_PHASE_PUSH_DEPOSIT, (int)ctx->sp.size());
                for (auto& sp : ctx->sp) PK<T>::boris_push(s, g, view<T>(sp), sp.q, sp.m, ctx->E, ctx->B);
            }
            {
                Phase ph(ctx, PIC_PHASE_FIELDS, 1);
                PK<T>::yee_b_half(s, g, ctx->E, ctx->B);
            }
            Phase ph(ctx, PIC_PHASE_PUSH_DEPOSIT, (int)ctx->sp.size());
            CK(cudaMemsetAsync(ctx->J, 0, sizeof(double) * 3 * g.N, s));
            for (auto& sp : ctx->sp) PK<T>::zigzag(s, g, view<T>(sp), sp.q, sp.m, sp.w, ctx->J);
        }
        {
            Phase ph(ctx, PIC_PHASE_FIELDS, 2 * ctx->cfg.smoothing_count + 1);
            pic_status st = smooth_current(ctx);
            if (st != PIC_OK) return st;
            PK<T>::yee_e(s, g, ctx->E, ctx->B, ctx->J, ctx->e_right);
        }
        CKL(ctx, "buneman step");
        if (g.wall) ctx->pending_compact = true;   // escaped particles (cell -1) until the next sort
        ctx->step++;
    }
    return PIC_OK;
}

// -------------------------------------------------------------- implicit
template <typename T>
pic_status implicit_moments(pic_ctx* ctx) {
    Phase ph(ctx, PIC_PHASE_MOMENTS, (int)ctx->sp.size() + (ctx->cfg.pressure_compat ? 6 : 2) + 1);
    cudaStream_t s = ctx->s;
    const GridP& g = ctx->g;
    const long long N = g.N;
    CK(cudaMemsetAsync(ctx->Jh, 0, sizeof(double) * 3 * N, s));
    CK(cudaMemsetAsync(ctx->mu, 0, sizeof(double) * 9 * N, s));
    CK(cudaMemsetAsync(ctx->rho, 0, sizeof(double) * N, s));
    CK(cudaMemsetAsync(ctx->Pi, 0, sizeof(double) * ctx->pi_len, s));
    const int compat = ctx->cfg.pressure_compat;
    // tiled shared-memory deposit when the particles are in tile order and
    // the pressure tensor goes to the particle's cells; halo of one cell when
    // the block fits in shared memory
    // right after a sort every particle is in its tile: no halo, and E, B
    // staged next to the accumulators; otherwise a one-cell halo for drift
    ImpBlock bk = PK<T>::implicit_block(g, ctx->tg, 0);
    bk.stage = 1;
    if (!ctx->fresh_sort || PK<T>::implicit_tile_smem(bk) > 227 * 1024) {
        bk = PK<T>::implicit_block(g, ctx->tg, 1);
        if (PK<T>::implicit_tile_smem(bk) > 227 * 1024) bk = PK<T>::implicit_block(g, ctx->tg, 0);
    }
    if (!compat && all_sorted(ctx) && PK<T>::implicit_tile_smem(bk) <= 227 * 1024) {
        ImpSpecies<T> S{};
        S.ns = (int)ctx->sp.size();
        for (int q = 0; q < S.ns; ++q) {
            S.p[q] = view<T>(ctx->sp[q]);
            S.q[q] = ctx->sp[q].q; S.m[q] = ctx->sp[q].m; S.w[q] = ctx->sp[q].w;
            S.off[q] = ctx->sp[q].off;
        }
        const T* Ef = (const T*)ctx->Ei;
        const T* Bf = (const T*)ctx->Bi;
        if (sizeof(T) == sizeof(float)) {   // FP32 copies of E^n and B^n for the FP32 gathers
            if (!ctx->fields32) CK(dalloc(&ctx->fields32, sizeof(float) * 6 * (size_t)N));
            PK<float>::to_real(s, ctx->Ei, ctx->fields32, 3 * N);
            PK<float>::to_real(s, ctx->Bi, ctx->fields32 + 3 * N, 3 * N);
            Ef = (const T*)ctx->fields32;
            Bf = (const T*)(ctx->fields32 + 3 * N);
        }
        Phase dep(ctx, PIC_PHASE_DEPOSIT, 0);
        PK<T>::implicit_deposit_tiled(s, g, ctx->tg, bk, S, Ef, Bf, ctx->Jh, ctx->mu, ctx->rho, ctx->Pi);
    } else {
        Phase dep(ctx, PIC_PHASE_DEPOSIT, 0);
        for (auto& sp : ctx->sp)
            PK<T>::implicit_deposit(s, g, view<T>(sp), sp.q, sp.m, sp.w, ctx->Ei, ctx->Bi, ctx->Jh, ctx->mu,
                                    ctx->rho, ctx->Pi, compat, ctx->ga);
    }
    if (g.wall) launch_wall_moments(s, g, ctx->Jh, ctx->mu, ctx->rho, ctx->Pi, compat ? 0 : 1);
    if (compat) {
        // one rank next to a wall folds nothing along x (momentum_exchange.cpp:1643-1670)
        for (int ax = g.wall ? 1 : 0; ax < 3; ++ax) launch_pi_fold_reference(s, ctx->Pi, ctx->ga, ax);
        launch_jg_build(s, g, ctx->ga, ctx->Jh, ctx->Pi, ctx->Jg, ctx->nex, ctx->ney, ctx->nez);
        launch_rho_ext_reference(s, g, ctx->Jg, ctx->nex, ctx->ney, ctx->nez, ctx->rho, ctx->rho_ext, ctx->ex, ctx->ey,
                                 ctx->ez);
        launch_jg_interior(s, g, ctx->Jg, ctx->nex, ctx->ney, ctx->nez, ctx->ga.gx, ctx->ga.gy, ctx->ga.gz, ctx->Jh);
    } else {
        launch_j_minus_divpi(s, g, ctx->Pi, ctx->Jh, ctx->Jg);
        CK(cudaMemcpyAsync(ctx->Jh, ctx->Jg, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, s));
        if (g.wall) launch_wall_zero_j(s, g, ctx->Jh);
        launch_rho_ext_periodic(s, g, ctx->Jh, ctx->rho, ctx->rho_ext, ctx->ex, ctx->ey, ctx->ez);
        pic_status st = smooth_moments(ctx);
        if (st != PIC_OK) return st;
    }
    launch_maxwell_rhs(s, g, ctx->Ei, ctx->Bi, ctx->Jh, ctx->rho_ext, ctx->ex, ctx->ey, ctx->rhs);
    if (g.wall) launch_wall_rhs(s, g, ctx->rho_ext, ctx->ex, ctx->ey, ctx->e_right, ctx->rhs);
    CKL(ctx, "implicit moments");
    ctx->moments_ready = true;
    ctx->mu_valid = true;
    return PIC_OK;
}

template <typename T>
pic_status implicit_move(pic_ctx* ctx) {
    // the tiled mover and its deferred pass, or one untiled launch per species
    Phase ph(ctx, PIC_PHASE_MOVER, all_sorted(ctx) ? 2 : (int)ctx->sp.size());
    bool tiled = false;
    if (all_sorted(ctx)) {
        ImpSpecies<T> S{};
        S.ns = (int)ctx->sp.size();
        for (int q = 0; q < S.ns; ++q) {
            S.p[q] = view<T>(ctx->sp[q]);
            S.q[q] = ctx->sp[q].q; S.m[q] = ctx->sp[q].m; S.w[q] = ctx->sp[q].w;
            S.off[q] = ctx->sp[q].off;
            S.defer[q] = ctx->sp[q].defer;
        }
        tiled = PK<T>::implicit_push_tiled(ctx->s, ctx->g, ctx->tg, S, ctx->Ei, ctx->Bi, ctx->Et);
    }
    if (!tiled)
        for (auto& sp : ctx->sp)
            PK<T>::implicit_push(ctx->s, ctx->g, view<T>(sp), sp.q, sp.m, ctx->Ei, ctx->Bi, ctx->Et);
    CKL(ctx, "implicit mover");
    ctx->fresh_sort = false;
    // the tile order stays valid: the tiled deposit and mover check every
    // particle's cell and take their halo or global path for drifted ones
    return PIC_OK;
}

pic_status check_species(pic_ctx* ctx, int sid) {
    if (sid < 0 || sid >= (int)ctx->sp.size()) return fail(ctx, PIC_ERR_ARG, "no such species");
    return PIC_OK;
}

pic_status ensure_stage(pic_ctx* ctx, long long len) {
    if (len <= ctx->stage_len) return PIC_OK;
    if (ctx->stage) cudaFree(ctx->stage);
    ctx->stage = nullptr;
    ctx->stage_len = 0;
    CK(dalloc(&ctx->stage, sizeof(double) * (size_t)len));
    ctx->stage_len = len;
    return PIC_OK;
}

constexpr long long kStageChunk = 1LL << 25;   // doubles per host transfer chunk

// Host arrays that kernels can address directly (pinned or registered memory
// under unified addressing): the conversion kernels read and write them over
// the host link, with no staging copy and no separate conversion pass.
bool device_addressable(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged) && a.devicePointer == p;
}

}  // namespace

// ========================================================================== C ABI
extern "C" {

pic_status pic_create(const pic_config* cfg, pic_ctx** out) {
    if (!cfg || !out) return PIC_ERR_ARG;
    *out = nullptr;
    const pic_config& c = *cfg;
    if (c.nx < 1 || c.ny < 1 || c.nz < 1 || !(c.dx > 0) || !(c.dy > 0) || !(c.dz > 0) || !(c.dt > 0)) return PIC_ERR_ARG;
    if (c.solver != PIC_SOLVER_BUNEMAN && c.solver != PIC_SOLVER_IMPLICIT) return PIC_ERR_ARG;
    if (c.particle_real != PIC_REAL_F32 && c.particle_real != PIC_REAL_F64) return PIC_ERR_ARG;
    if (c.solver == PIC_SOLVER_BUNEMAN && c.field_real != c.particle_real) return PIC_ERR_ARG;
    if (c.solver == PIC_SOLVER_IMPLICIT && !(c.theta > 0)) return PIC_ERR_ARG;
    if (c.smoothing_count < 0 || (c.smoothing_count > 0 && !(c.smoothing_parameter >= 0 && c.smoothing_parameter <= 1)))
        return PIC_ERR_ARG;
    // the reference smooths J-hat and rho-hat including its own ghost values,
    // which only the periodic pressure placement represents as periodic images
    if (c.smoothing_count > 0 && c.solver == PIC_SOLVER_IMPLICIT && c.pressure_compat) return PIC_ERR_ARG;
    // conductor wall / open boundary along x: 3-D boxes, no smoothing (the
    // reference's own 2-D boundary rows are all fake, fields.cpp:528-530);
    // explicit runs reflect at node kTristanWallNode, so their box reaches
    // at least four cells beyond it
    if (c.boundary_x != PIC_BOUNDARY_PERIODIC &&
        (c.boundary_x != PIC_BOUNDARY_WALL_OPEN || c.smoothing_count > 0 || c.ny < 2 || c.nz < 2 ||
         c.nx < (c.solver == PIC_SOLVER_BUNEMAN ? kTristanWallNode + 6 : 4)))
        return PIC_ERR_ARG;
    long long N = (long long)c.nx * c.ny * c.nz;
    if (N >= (1LL << 31)) return PIC_ERR_ARG;
    int tile[3];
    const int n3[3] = {c.nx, c.ny, c.nz};
    for (int a = 0; a < 3; ++a) {
        int t = c.tile[a];
        if (t <= 0) {   // default: the largest of 8, 4, 2, 1 dividing the axis
            t = 8;
            while (t > 1 && n3[a] % t != 0) t /= 2;
        }
        if (t > n3[a]) t = n3[a];
        if (n3[a] % t != 0) return PIC_ERR_ARG;
        tile[a] = t;
    }
    pic_ctx* ctx = new pic_ctx();
    ctx->cfg = c;
    if (ctx->cfg.max_species <= 0) ctx->cfg.max_species = kMaxSpecies;
    if (ctx->cfg.max_species > kMaxSpecies) { delete ctx; return PIC_ERR_ARG; }
    if (ctx->cfg.cfix == 0) ctx->cfg.cfix = 1.025;
    GridP& g = ctx->g;
    g.nx = c.nx; g.ny = c.ny; g.nz = c.nz; g.N = N;
    g.dx = c.dx; g.dy = c.dy; g.dz = c.dz; g.dt = c.dt;
    g.idx = 1.0 / c.dx; g.idy = 1.0 / c.dy; g.idz = 1.0 / c.dz;
    g.theta = c.theta; g.eta = c.eta; g.cfix = ctx->cfg.cfix;
    g.y3 = c.ny > 1; g.z3 = c.nz > 1;
    g.divx = FastDiv((unsigned)c.nx);
    g.divy = FastDiv((unsigned)c.ny);
    g.wall = c.boundary_x == PIC_BOUNDARY_WALL_OPEN ? 1 : 0;
    for (int a = 0; a < 3; ++a) { ctx->e_right[a] = c.e_right[a]; ctx->b_right[a] = c.b_right[a]; }
    ctx->preal = c.particle_real;
    ctx->rsz = ctx->preal ? sizeof(double) : sizeof(float);
    TileGeom& t = ctx->tg;
    t.tx = tile[0]; t.ty = tile[1]; t.tz = tile[2];
    t.ntx = c.nx / t.tx; t.nty = c.ny / t.ty; t.ntz = c.nz / t.tz;
    {
        auto lg = [](int v) { int l = 0; while ((1 << l) < v) ++l; return (1 << l) == v ? l : -1; };
        t.lx = lg(t.tx); t.ly = lg(t.ty); t.lz = lg(t.tz);
        if (t.lx < 0 || t.ly < 0 || t.lz < 0) t.lx = t.ly = t.lz = -1;
    }
    ctx->ntiles = t.ntx * t.nty * t.ntz;
    ctx->T3 = t.tx * t.ty * t.tz;
    ctx->nkeys = (int)N;
    TileShape& ts = ctx->ts;
    ts.hx = 2; ts.hy = g.y3 ? 2 : 0; ts.hz = g.z3 ? 2 : 0;
    ts.gx = 2; ts.gy = g.y3 ? 2 : 0; ts.gz = g.z3 ? 2 : 0;
    ts.fx = t.tx + 2 * ts.hx; ts.fy = t.ty + 2 * ts.hy; ts.fz = t.tz + 2 * ts.hz;
    ts.jx = t.tx + 2 * ts.gx; ts.jy = t.ty + 2 * ts.gy; ts.jz = t.tz + 2 * ts.gz;
    ts.jcells = (long long)ts.jx * ts.jy * ts.jz;
    // the fused explicit kernel holds the tile's fields and current in shared memory
    if (c.solver == PIC_SOLVER_BUNEMAN &&
        (ctx->preal ? PK<double>::tile_smem_bytes(ts) : PK<float>::tile_smem_bytes(ts)) > 200 * 1024) {
        delete ctx;
        return PIC_ERR_ARG;
    }
    GhostAxes& ga = ctx->ga;
    ga.cex = c.nx > 1 ? c.nx + 4 : 1; ga.cey = c.ny > 1 ? c.ny + 4 : 1; ga.cez = c.nz > 1 ? c.nz + 4 : 1;
    ga.gx = c.nx > 1 ? 2 : 0; ga.gy = c.ny > 1 ? 2 : 0; ga.gz = c.nz > 1 ? 2 : 0;
    ctx->nex = c.nx > 1 ? c.nx + 5 : 1; ctx->ney = c.ny > 1 ? c.ny + 5 : 1; ctx->nez = c.nz > 1 ? c.nz + 5 : 1;
    ctx->ex = c.nx > 1 ? c.nx + 1 : 1; ctx->ey = c.ny > 1 ? c.ny + 1 : 1; ctx->ez = c.nz > 1 ? c.nz + 1 : 1;

    cudaError_t e = cudaStreamCreateWithFlags(&ctx->s, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete ctx; return PIC_ERR_CUDA; }
    auto A = [&](auto** p, size_t bytes) -> bool {
        cudaError_t r = dalloc(p, bytes);
        if (r != cudaSuccess) { ctx->err = cudaGetErrorString(r); return false; }
        return cudaMemsetAsync(*p, 0, bytes, ctx->s) == cudaSuccess;
    };
    bool ok = true;
    ok = ok && A(&ctx->counts, sizeof(int) * ((size_t)N + 1));
    ok = ok && A(&ctx->cursor, sizeof(int) * (size_t)N);
    ok = ok && A(&ctx->block_sums, sizeof(int) * (size_t)(N / 2048 + 2));
    ok = ok && A(&ctx->long_count, sizeof(int));
    ok = ok && A(&ctx->partials, sizeof(double) * 8 * 1024);
    ok = ok && A(&ctx->flag, sizeof(int));
    if (c.solver == PIC_SOLVER_BUNEMAN) {
        ok = ok && A(&ctx->E, ctx->rsz * 3 * N);
        ok = ok && A(&ctx->B, ctx->rsz * 3 * N);
        ok = ok && A(&ctx->J, sizeof(double) * 3 * N);
        ok = ok && A(&ctx->Jfix, sizeof(double) * 3 * N);
        ok = ok && A(&ctx->Jpart, sizeof(double) * 3 * (size_t)ts.jcells * ctx->ntiles);
    } else {
        ctx->pi_len = c.pressure_compat ? 9LL * ga.cex * ga.cey * ga.cez : 9 * N;
        ctx->jg_len = c.pressure_compat ? 3LL * ctx->nex * ctx->ney * ctx->nez : 3 * N;
        ctx->rho_ext_len = (long long)ctx->ex * ctx->ey * ctx->ez;
        ok = ok && A(&ctx->Ei, sizeof(double) * 3 * N);
        ok = ok && A(&ctx->Bi, sizeof(double) * 3 * N);
        ok = ok && A(&ctx->Jh, sizeof(double) * 3 * N);
        ok = ok && A(&ctx->mu, sizeof(double) * 9 * N);
        ok = ok && A(&ctx->rho, sizeof(double) * N);
        ok = ok && A(&ctx->rho_ext, sizeof(double) * ctx->rho_ext_len);
        ok = ok && A(&ctx->Pi, sizeof(double) * ctx->pi_len);
        ok = ok && A(&ctx->Jg, sizeof(double) * ctx->jg_len);
        ok = ok && A(&ctx->rhs, sizeof(double) * 3 * N);
        ok = ok && A(&ctx->Et, sizeof(double) * 3 * N);
        ok = ok && A(&ctx->En, sizeof(double) * 3 * N);
        ok = ok && A(&ctx->Bn, sizeof(double) * 3 * N);
    }
    if (ok) ok = ensure_stage(ctx, std::max<long long>(3 * N, 1 << 20)) == PIC_OK;
    if (ok) ok = cudaStreamSynchronize(ctx->s) == cudaSuccess;
    if (!ok) {
        pic_destroy(ctx);
        return PIC_ERR_NOMEM;
    }
    *out = ctx;
    return PIC_OK;
}

pic_status pic_destroy(pic_ctx* ctx) {
    if (!ctx) return PIC_OK;
    if (ctx->s) cudaStreamSynchronize(ctx->s);
    for (auto& sp : ctx->sp) {
        cudaFree(sp.cell); cudaFree(sp.id); cudaFree(sp.cell2); cudaFree(sp.id2);
        for (int q = 0; q < 6; ++q) { cudaFree(sp.a[q]); cudaFree(sp.b[q]); }
        cudaFree(sp.perm); cudaFree(sp.off); cudaFree(sp.defer);
    }
    void* bufs[] = {ctx->E, ctx->B, ctx->J, ctx->Jfix, ctx->Jpart, ctx->Ei, ctx->Bi, ctx->Jh, ctx->mu, ctx->rho,
                    ctx->rho_ext, ctx->Pi, ctx->Jg, ctx->rhs, ctx->Et, ctx->En, ctx->Bn, ctx->key, ctx->counts,
                    ctx->cursor, ctx->tmp, ctx->block_sums, ctx->long_count, ctx->long_list, ctx->stage,
                    ctx->partials, ctx->flag};
    for (void* b : bufs) if (b) cudaFree(b);
    krylov_free(ctx->kry);
    delete ctx->net;
    cudaFree(ctx->dens);
    cudaFree(ctx->dens_rho);
    cudaFree(ctx->smooth_tmp);
    cudaFree(ctx->fields32);
    if (ctx->s) cudaStreamDestroy(ctx->s);
    delete ctx;
    return PIC_OK;
}

const char* pic_last_error(const pic_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void* pic_stream(pic_ctx* ctx) { return ctx ? (void*)ctx->s : nullptr; }

pic_status pic_add_species(pic_ctx* ctx, double q, double m, double w, long capacity, int* species_id) {
    if (!ctx) return PIC_ERR_ARG;
    if ((int)ctx->sp.size() >= ctx->cfg.max_species) return fail(ctx, PIC_ERR_ARG, "too many species");
    if (!(m > 0) || capacity < 0 || capacity >= (1L << 31) || !std::isfinite(q) || !std::isfinite(w))
        return fail(ctx, PIC_ERR_ARG, "bad species parameters");
    Species sp;
    sp.q = q; sp.m = m; sp.w = w; sp.cap = capacity;
    const size_t n = (size_t)std::max<long>(capacity, 1);
    CK(dalloc(&sp.cell, sizeof(int) * n));
    CK(dalloc(&sp.id, sizeof(int) * n));
    CK(dalloc(&sp.cell2, sizeof(int) * n));
    CK(dalloc(&sp.id2, sizeof(int) * n));
    for (int a = 0; a < 6; ++a) {
        CK(dalloc(&sp.a[a], ctx->rsz * n));
        CK(dalloc(&sp.b[a], ctx->rsz * n));
    }
    CK(dalloc(&sp.perm, sizeof(int) * n));
    // one bit per particle and kind, plus the word a chunk that starts in the
    // last one spills into; zero between steps (the deferred pass clears
    // what it reads)
    sp.dwords = ((long long)n + 31) / 32 + 1;
    CK(dalloc(&sp.defer, sizeof(unsigned) * 2 * (size_t)sp.dwords));
    CK(cudaMemsetAsync(sp.defer, 0, sizeof(unsigned) * 2 * (size_t)sp.dwords, ctx->s));
    CK(dalloc(&sp.off, sizeof(int) * ((size_t)ctx->nkeys + 1)));
    CK(cudaMemsetAsync(sp.off, 0, sizeof(int) * ((size_t)ctx->nkeys + 1), ctx->s));
    if ((long long)n > ctx->sort_cap) {
        cudaFree(ctx->key); cudaFree(ctx->tmp); cudaFree(ctx->long_list);
        CK(dalloc(&ctx->key, sizeof(int) * n));
        CK(dalloc(&ctx->tmp, sizeof(int) * n));
        CK(dalloc(&ctx->long_list, sizeof(int) * ((size_t)ctx->nkeys + 1)));
        ctx->sort_cap = (long long)n;
    }
    ctx->sp.push_back(sp);
    if (species_id) *species_id = (int)ctx->sp.size() - 1;
    return sync(ctx, "add species");
}

namespace {

// Host particles into slots [at, at + n) of a species (upload: at = 0, the
// species then holds n; append: at = its count), validated on the device.
pic_status put_particles(pic_ctx* ctx, int sid, long long at, long n, const int* cell, const double* ox,
                         const double* oy, const double* oz, const double* px, const double* py, const double* pz,
                         const int* ids) {
    Species& sp = ctx->sp[sid];
    if (n < 0 || at + n > sp.cap) return fail(ctx, PIC_ERR_NOMEM, "particle count exceeds species capacity");
    if (n > 0 && (!cell || !ox || !oy || !oz || !px || !py || !pz)) return fail(ctx, PIC_ERR_ARG, "null array");
    const long long n0 = sp.n;
    cudaStream_t s = ctx->s;
    CK(cudaMemcpyAsync(sp.cell + at, cell, sizeof(int) * n, cudaMemcpyHostToDevice, s));
    if (ids) {
        CK(cudaMemcpyAsync(sp.id + at, ids, sizeof(int) * n, cudaMemcpyHostToDevice, s));
    } else {
        PK<float>::iota(s, sp.id + at, n, at == 0 ? 0 : sp.next_id);
    }
    const double* src[6] = {ox, oy, oz, px, py, pz};
    const long long chunk = std::min<long long>(kStageChunk, ctx->stage_len);
    // validation on the device: cell range, offsets in [0,1), finite momenta;
    // FP32 conversion checks the FP64 values before rounding
    CK(cudaMemsetAsync(ctx->flag, 0, sizeof(int), s));
    for (int q = 0; q < 6; ++q) {
        if (ctx->preal) {
            CK(cudaMemcpyAsync((double*)sp.a[q] + at, src[q], sizeof(double) * n, cudaMemcpyHostToDevice, s));
            continue;
        }
        if (device_addressable(src[q])) {
            PK<float>::to_real_checked(s, src[q], (float*)sp.a[q] + at, n, q < 3 ? 0 : 1, ctx->flag);
            continue;
        }
        for (long long b = 0; b < n; b += chunk) {
            long long len = std::min<long long>(chunk, n - b);
            CK(cudaMemcpyAsync(ctx->stage, src[q] + b, sizeof(double) * len, cudaMemcpyHostToDevice, s));
            PK<float>::to_real_checked(s, ctx->stage, (float*)sp.a[q] + at + b, len, q < 3 ? 0 : 1, ctx->flag);
        }
    }
    // validate the new slots only
    Species part = sp;
    for (int q = 0; q < 6; ++q) part.a[q] = (char*)sp.a[q] + ctx->rsz * at;
    part.cell = sp.cell + at;
    part.n = n;
    if (ctx->preal) PK<double>::validate(s, ctx->g, view<double>(part), ctx->flag);
    else PK<float>::validate(s, ctx->g, view<float>(part), ctx->flag);
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, ctx->flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (bad) {
        sp.n = at == 0 ? 0 : n0;
        if (bad & 4) return fail(ctx, PIC_ERR_NUMERIC, "non-finite particle momentum");
        return fail(ctx, PIC_ERR_ARG, (bad & 1) ? "cell index out of range" : "offset outside [0,1)");
    }
    sp.n = at + n;
    sp.next_id = at == 0 ? n : sp.next_id + n;
    sp.sorted = false;
    ctx->moments_ready = false;
    return sync(ctx, "put particles");
}

}  // namespace

pic_status pic_upload_particles(pic_ctx* ctx, int sid, long n, const int* cell, const double* ox, const double* oy,
                                const double* oz, const double* px, const double* py, const double* pz,
                                const int* ids) {
    if (!ctx) return PIC_ERR_ARG;
    if (pic_status st = check_species(ctx, sid)) return st;
    return put_particles(ctx, sid, 0, n, cell, ox, oy, oz, px, py, pz, ids);
}

pic_status pic_append_particles(pic_ctx* ctx, int sid, long n, const int* cell, const double* ox, const double* oy,
                                const double* oz, const double* px, const double* py, const double* pz,
                                const int* ids) {
    if (!ctx) return PIC_ERR_ARG;
    if (pic_status st = check_species(ctx, sid)) return st;
    if (pic_status st = settle(ctx)) return st;
    return put_particles(ctx, sid, ctx->sp[sid].n, n, cell, ox, oy, oz, px, py, pz, ids);
}

pic_status pic_fill_species(pic_ctx* ctx, int sid, int ppc, unsigned long long seed, double theta, double drift_gamma,
                            int alternate_drift) {
    if (!ctx) return PIC_ERR_ARG;
    if (pic_status st = check_species(ctx, sid)) return st;
    Species& sp = ctx->sp[sid];
    if (ppc < 0 || !(theta >= 0) || !(drift_gamma >= 1.0)) return fail(ctx, PIC_ERR_ARG, "bad fill parameters");
    // a wall box leaves its two ghost columns empty; the explicit path fills
    // from its reflecting wall on (createParticles, initialization.cpp
    // 8152-8155)
    const int x0 = ctx->g.wall && is_buneman(ctx) ? kTristanWallNode : 0;
    const int rowx = ctx->g.wall ? ctx->g.nx - 2 - x0 : ctx->g.nx;
    const long long n = (long long)ppc * (ctx->g.N / ctx->g.nx) * rowx;
    if (n > sp.cap) return fail(ctx, PIC_ERR_NOMEM, "particle count exceeds species capacity");
    const int ntab = 4096;
    std::vector<double> us, cdf;
    if (theta > 0) cdf = juttner_table(theta, ntab, us);
    double* du = ctx->stage;
    double* dc = ctx->stage + ntab;
    if (theta > 0) {
        CK(cudaMemcpyAsync(du, us.data(), sizeof(double) * ntab, cudaMemcpyHostToDevice, ctx->s));
        CK(cudaMemcpyAsync(dc, cdf.data(), sizeof(double) * ntab, cudaMemcpyHostToDevice, ctx->s));
    }
    sp.n = n;
    const unsigned long long sseed = seed * 0x100000001B3ull + (unsigned long long)sid * 0x9E3779B97F4A7C15ull;
    if (ctx->preal) launch_fill<double>(ctx->s, view<double>(sp), ppc, sseed, du, dc, theta > 0 ? ntab : 0, sp.m,
                                        drift_gamma, alternate_drift, rowx, ctx->g.nx, x0);
    else launch_fill<float>(ctx->s, view<float>(sp), ppc, sseed, du, dc, theta > 0 ? ntab : 0, sp.m, drift_gamma,
                            alternate_drift, rowx, ctx->g.nx, x0);
    CKL(ctx, "fill species");
    sp.next_id = n;
    sp.sorted = false;
    ctx->moments_ready = false;
    return sync(ctx, "fill species");
}

pic_status pic_download_particles(pic_ctx* ctx, int sid, long* n_out, int* cell, double* ox, double* oy, double* oz,
                                  double* px, double* py, double* pz, int* ids) {
    if (!ctx) return PIC_ERR_ARG;
    if (pic_status st = check_species(ctx, sid)) return st;
    if (pic_status st0 = settle(ctx)) return st0;
    Species& sp = ctx->sp[sid];
    const long long n = sp.n;
    if (n_out) *n_out = (long)n;
    cudaStream_t s = ctx->s;
    if (cell) CK(cudaMemcpyAsync(cell, sp.cell, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    if (ids) CK(cudaMemcpyAsync(ids, sp.id, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    double* dst[6] = {ox, oy, oz, px, py, pz};
    const long long chunk = std::min<long long>(kStageChunk, ctx->stage_len);
    for (int q = 0; q < 6; ++q) {
        if (!dst[q]) continue;
        if (ctx->preal) {
            CK(cudaMemcpyAsync(dst[q], sp.a[q], sizeof(double) * n, cudaMemcpyDeviceToHost, s));
            continue;
        }
        if (device_addressable(dst[q])) {
            PK<float>::from_real(s, sp.a[q], dst[q], n);
            continue;
        }
        // staged: the stream orders each conversion after the previous copy out of the stage
        for (long long b = 0; b < n; b += chunk) {
            long long len = std::min<long long>(chunk, n - b);
            PK<float>::from_real(s, (float*)sp.a[q] + b, ctx->stage, len);
            CK(cudaMemcpyAsync(dst[q] + b, ctx->stage, sizeof(double) * len, cudaMemcpyDeviceToHost, s));
        }
    }
    return sync(ctx, "download particles");
}

pic_status pic_upload_fields(pic_ctx* ctx, const double* E, const double* B) {
    if (!ctx) return PIC_ERR_ARG;
    const long long L = 3 * ctx->g.N;
    cudaStream_t s = ctx->s;
    const double* src[2] = {E, B};
    // each field goes to the stage buffer (3N doubles) and is checked there
    // on the device: a non-finite value rejects it before the state changes
    for (int f = 0; f < 2; ++f) {
        if (!src[f]) continue;
        CK(cudaMemcpyAsync(ctx->stage, src[f], sizeof(double) * L, cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(ctx->flag, 0, sizeof(int), s));
        launch_nonfinite(s, ctx->stage, L, ctx->flag);
        int bad = 0;
        CK(cudaMemcpyAsync(&bad, ctx->flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (bad) return fail(ctx, PIC_ERR_NUMERIC, "non-finite field value");
        if (is_buneman(ctx)) {
            void* dst = f == 0 ? ctx->E : ctx->B;
            if (ctx->preal) CK(cudaMemcpyAsync(dst, ctx->stage, sizeof(double) * L, cudaMemcpyDeviceToDevice, s));
            else PK<float>::to_real(s, ctx->stage, dst, L);
        } else {
            CK(cudaMemcpyAsync(f == 0 ? ctx->Ei : ctx->Bi, ctx->stage, sizeof(double) * L, cudaMemcpyDeviceToDevice, s));
        }
    }
    ctx->moments_ready = false;
    return sync(ctx, "upload fields");
}

pic_status pic_download_fields(pic_ctx* ctx, double* E, double* B, double* J) {
    if (!ctx) return PIC_ERR_ARG;
    const long long L = 3 * ctx->g.N;
    cudaStream_t s = ctx->s;
    double* dst[2] = {E, B};
    for (int f = 0; f < 2; ++f) {
        if (!dst[f]) continue;
        if (is_buneman(ctx)) {
            void* src = f == 0 ? ctx->E : ctx->B;
            if (ctx->preal) {
                CK(cudaMemcpyAsync(dst[f], src, sizeof(double) * L, cudaMemcpyDeviceToHost, s));
            } else if (device_addressable(dst[f])) {
                PK<float>::from_real(s, src, dst[f], L);
            } else {
                PK<float>::from_real(s, src, ctx->stage, L);
                CK(cudaMemcpyAsync(dst[f], ctx->stage, sizeof(double) * L, cudaMemcpyDeviceToHost, s));
            }
        } else {
            CK(cudaMemcpyAsync(dst[f], f == 0 ? ctx->Ei : ctx->Bi, sizeof(double) * L, cudaMemcpyDeviceToHost, s));
        }
    }
    if (J) CK(cudaMemcpyAsync(J, is_buneman(ctx) ? ctx->J : ctx->Jh, sizeof(double) * L, cudaMemcpyDeviceToHost, s));
    return sync(ctx, "download fields");
}

// ---------------------------------------------------------------- explicit phases
pic_status pic_tristan_evaluate_b_half_step(pic_ctx* ctx) {
    if (!ctx) return PIC_ERR_ARG;
    if (!is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not a Buneman run");
    if (ctx->preal) PK<double>::yee_b_half(ctx->s, ctx->g, ctx->E, ctx->B);
    else PK<float>::yee_b_half(ctx->s, ctx->g, ctx->E, ctx->B);
    return sync(ctx, "b half step");
}

pic_status pic_move_particles(pic_ctx* ctx) {
    if (!ctx) return PIC_ERR_ARG;
    if (is_buneman(ctx)) {
        for (auto& sp : ctx->sp) {
            if (ctx->preal) PK<double>::boris_push(ctx->s, ctx->g, view<double>(sp), sp.q, sp.m, ctx->E, ctx->B);
            else PK<float>::boris_push(ctx->s, ctx->g, view<float>(sp), sp.q, sp.m, ctx->E, ctx->B);
            sp.sorted = false;
        }
        // escaped particles deposit their current (pic_tristan_update_flux),
        // which marks them; the next sort erases them
        if (ctx->g.wall) ctx->pending_compact = true;
        return sync(ctx, "move particles");
    }
    if (!ctx->efield_ready) return fail(ctx, PIC_ERR_STATE, "evaluate the electric field first");
    pic_status st = ctx->preal ? implicit_move<double>(ctx) : implicit_move<float>(ctx);
    if (st != PIC_OK) return st;
    if (ctx->g.wall) ctx->pending_compact = true;   // escaped particles are erased by the next sort
    return sync(ctx, "move particles");
}

pic_status pic_tristan_update_flux(pic_ctx* ctx) {
    if (!ctx) return PIC_ERR_ARG;
    if (!is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not a Buneman run");
    CK(cudaMemsetAsync(ctx->J, 0, sizeof(double) * 3 * ctx->g.N, ctx->s));
    for (auto& sp : ctx->sp) {
        if (ctx->preal) PK<double>::zigzag(ctx->s, ctx->g, view<double>(sp), sp.q, sp.m, sp.w, ctx->J);
        else PK<float>::zigzag(ctx->s, ctx->g, view<float>(sp), sp.q, sp.m, sp.w, ctx->J);
    }
    pic_status st = smooth_current(ctx);
    if (st != PIC_OK) return st;
    return sync(ctx, "update flux");
}

pic_status pic_tristan_evaluate_e(pic_ctx* ctx) {
    if (!ctx) return PIC_ERR_ARG;
    if (!is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not a Buneman run");
    if (ctx->preal) PK<double>::yee_e(ctx->s, ctx->g, ctx->E, ctx->B, ctx->J, ctx->e_right);
    else PK<float>::yee_e(ctx->s, ctx->g, ctx->E, ctx->B, ctx->J, ctx->e_right);
    return sync(ctx, "evaluate E");
}

pic_status pic_buneman_step(pic_ctx* ctx, int nsteps) {
    if (!ctx || nsteps < 0) return PIC_ERR_ARG;
    if (!is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not a Buneman run");
    pic_status st = ctx->preal ? buneman_steps<double>(ctx, nsteps) : buneman_steps<float>(ctx, nsteps);
    if (st != PIC_OK) return st;
    return sync(ctx, "buneman step");
}

// ---------------------------------------------------------------- implicit phases
pic_status pic_update_electromagnetic_parameters(pic_ctx* ctx) {
    if (!ctx) return PIC_ERR_ARG;
    if (is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not an implicit run");
    if (ctx->pending_compact ||
        (ctx->cfg.sort_every > 0 && (!all_sorted(ctx) || ctx->step % ctx->cfg.sort_every == 0))) {
        pic_status st = sort_all(ctx);
        if (st != PIC_OK) return st;
    }
    pic_status st = ctx->preal ? implicit_moments<double>(ctx) : implicit_moments<float>(ctx);
    if (st != PIC_OK) return st;
    return sync(ctx, "electromagnetic parameters");
}

static pic_status solve_into(pic_ctx* ctx, const double* mu, const double* rhs, double* x, const pic_solve_opts* o,
                             pic_solve_info* info) {
    pic_solve_opts d{PIC_GMRES_REFERENCE, 30, 50, 1e-8};
    const pic_solve_opts& opts = o ? *o : d;
    SolveCtx sc{ctx->s, &ctx->g, mu, ctx->partials, ctx->flag, &ctx->kry, &ctx->err, ctx->net};
    return krylov_solve(sc, rhs, x, opts, info);
}

pic_status pic_evaluate_electric_field(pic_ctx* ctx, const pic_solve_opts* opts, pic_solve_info* info) {
    if (!ctx) return PIC_ERR_ARG;
    if (is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not an implicit run");
    if (!ctx->moments_ready) return fail(ctx, PIC_ERR_STATE, "update the electromagnetic parameters first");
    pic_status st;
    {
        Phase ph(ctx, PIC_PHASE_SOLVE, 0);
        st = solve_into(ctx, ctx->mu, ctx->rhs, ctx->Et, opts, info);
        if (ctx->prof_on && info) ctx->launches += 6L * info->iterations + 8;
    }
    if (st != PIC_OK && st != PIC_ERR_NOT_CONVERGED) return st;
    const int method = opts ? opts->method : PIC_GMRES_REFERENCE;
    if (st == PIC_OK && ctx->trip.data && (method == PIC_GMRES_REFERENCE || method == PIC_GMRES_RESTARTED)) {
        pic_status rs = ctx->trip.add(ctx->s, ctx->rhs, ctx->mu, ctx->Et, ctx->partials + 7 * 1024, ctx->partials,
                                      &ctx->err);
        if (rs != PIC_OK) return rs;
    }
    {
        Phase ph(ctx, PIC_PHASE_FIELDS, 1);
        launch_field_update(ctx->s, ctx->g, ctx->Et, ctx->Ei, ctx->Bi, ctx->En, ctx->Bn, 1, 0);
    }
    ctx->efield_ready = true;
    pic_status s2 = sync(ctx, "evaluate electric field");
    return s2 != PIC_OK ? s2 : st;
}

pic_status pic_evaluate_magnetic_field(pic_ctx* ctx) {
    if (!ctx) return PIC_ERR_ARG;
    if (is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not an implicit run");
    if (!ctx->efield_ready) return fail(ctx, PIC_ERR_STATE, "evaluate the electric field first");
    {
        Phase ph(ctx, PIC_PHASE_FIELDS, 1);
        launch_field_update(ctx->s, ctx->g, ctx->Et, ctx->Ei, ctx->Bi, ctx->En, ctx->Bn, 0, 1);
        if (ctx->g.wall) launch_wall_b(ctx->s, ctx->g, ctx->Bn, ctx->b_right);
    }
    return sync(ctx, "evaluate magnetic field");
}

pic_status pic_update_fields(pic_ctx* ctx) {
    if (!ctx) return PIC_ERR_ARG;
    if (is_buneman(ctx)) return PIC_OK;   // the Yee grids are updated in place
    if (!ctx->efield_ready) return fail(ctx, PIC_ERR_STATE, "evaluate the fields first");
    std::swap(ctx->Ei, ctx->En);
    std::swap(ctx->Bi, ctx->Bn);
    ctx->efield_ready = false;
    ctx->moments_ready = false;
    ctx->step++;
    return PIC_OK;
}

pic_status pic_implicit_step(pic_ctx* ctx, const pic_solve_opts* opts, pic_solve_info* info) {
    pic_status st = pic_update_electromagnetic_parameters(ctx);
    if (st != PIC_OK) return st;
    pic_status solve = pic_evaluate_electric_field(ctx, opts, info);
    if (solve != PIC_OK && solve != PIC_ERR_NOT_CONVERGED) return solve;
    if ((st = pic_evaluate_magnetic_field(ctx)) != PIC_OK) return st;
    if ((st = pic_move_particles(ctx)) != PIC_OK) return st;
    if ((st = pic_update_fields(ctx)) != PIC_OK) return st;
    return solve;
}

pic_status pic_download_moments(pic_ctx* ctx, double* J, double* mu, double* rho_ext, double* rhs) {
    if (!ctx) return PIC_ERR_ARG;
    if (is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not an implicit run");
    const long long N = ctx->g.N;
    cudaStream_t s = ctx->s;
    if (J) CK(cudaMemcpyAsync(J, ctx->Jh, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s));
    if (mu) CK(cudaMemcpyAsync(mu, ctx->mu, sizeof(double) * 9 * N, cudaMemcpyDeviceToHost, s));
    if (rho_ext) CK(cudaMemcpyAsync(rho_ext, ctx->rho_ext, sizeof(double) * ctx->rho_ext_len, cudaMemcpyDeviceToHost, s));
    if (rhs) CK(cudaMemcpyAsync(rhs, ctx->rhs, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s));
    return sync(ctx, "download moments");
}

pic_status pic_maxwell_apply(pic_ctx* ctx, const double* mu, const double* x, double* y) {
    if (!ctx || !mu || !x || !y) return PIC_ERR_ARG;
    if (is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not an implicit run");
    const long long N = ctx->g.N;
    cudaStream_t s = ctx->s;
    CK(cudaMemcpyAsync(ctx->mu, mu, sizeof(double) * 9 * N, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->Et, x, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s));
    OpCoef oc = make_opcoef(ctx->g);
    pic_status st = ensure_smooth_tmp(ctx);
    if (st != PIC_OK) return st;
    launch_maxwell_apply(s, ctx->g, oc, ctx->mu, ctx->Et, ctx->En, ctx->smooth_tmp);
    CK(cudaMemcpyAsync(y, ctx->En, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s));
    ctx->mu_valid = true;
    ctx->moments_ready = false;
    ctx->efield_ready = false;
    return sync(ctx, "maxwell apply");
}

pic_status pic_maxwell_apply_transpose(pic_ctx* ctx, const double* mu, const double* y, double* out) {
    if (!ctx || !mu || !y || !out) return PIC_ERR_ARG;
    if (is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not an implicit run");
    if (ctx->g.wall) return fail(ctx, PIC_ERR_STATE, "the transpose covers periodic boxes only");
    const long long N = ctx->g.N;
    cudaStream_t s = ctx->s;
    CK(cudaMemcpyAsync(ctx->mu, mu, sizeof(double) * 9 * N, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->Et, y, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s));
    OpCoef oc = make_opcoef(ctx->g);
    launch_maxwell_apply_t(s, ctx->g, oc, ctx->mu, ctx->Et, ctx->En);
    CK(cudaMemcpyAsync(out, ctx->En, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s));
    ctx->mu_valid = true;
    ctx->moments_ready = false;
    ctx->efield_ready = false;
    return sync(ctx, "maxwell apply transpose");
}

pic_status pic_maxwell_solve(pic_ctx* ctx, const double* mu, const double* rhs, double* x, const pic_solve_opts* opts,
                             pic_solve_info* info) {
    if (!ctx || !mu || !rhs || !x) return PIC_ERR_ARG;
    if (is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not an implicit run");
    const long long N = ctx->g.N;
    cudaStream_t s = ctx->s;
    CK(cudaMemcpyAsync(ctx->mu, mu, sizeof(double) * 9 * N, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->rhs, rhs, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s));
    ctx->mu_valid = true;
    pic_status st = solve_into(ctx, ctx->mu, ctx->rhs, ctx->Et, opts, info);
    if (st != PIC_OK && st != PIC_ERR_NOT_CONVERGED) return st;
    CK(cudaMemcpyAsync(x, ctx->Et, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s));
    ctx->moments_ready = false;
    ctx->efield_ready = false;
    pic_status s2 = sync(ctx, "maxwell solve");
    return s2 != PIC_OK ? s2 : st;
}

pic_status pic_sort_particles(pic_ctx* ctx) {
    if (!ctx) return PIC_ERR_ARG;
    pic_status st = sort_all(ctx);
    if (st != PIC_OK) return st;
    return sync(ctx, "sort");
}

pic_status pic_download_permutation(pic_ctx* ctx, int sid, long* n, int* perm) {
    if (!ctx) return PIC_ERR_ARG;
    if (pic_status st = check_species(ctx, sid)) return st;
    Species& sp = ctx->sp[sid];
    if (n) *n = (long)sp.n;
    if (perm) CK(cudaMemcpyAsync(perm, sp.perm, sizeof(int) * sp.n, cudaMemcpyDeviceToHost, ctx->s));
    return sync(ctx, "download permutation");
}

pic_status pic_energy(pic_ctx* ctx, double out[6]) {
    if (!ctx || !out) return PIC_ERR_ARG;
    if (pic_status st0 = settle(ctx)) return st0;
    cudaStream_t s = ctx->s;
    const long long L = 3 * ctx->g.N;
    const double vol = ctx->g.dx * ctx->g.dy * ctx->g.dz;
    const double pi = 3.14159265358979323846;
    for (int q = 0; q < 6; ++q) out[q] = 0;
    std::vector<double> h(4 * 1024);
    for (auto& sp : ctx->sp) {
        const int P = red_blocks(sp.n);
        if (ctx->preal) PK<double>::particle_sums(s, view<double>(sp), sp.m, sp.w, ctx->partials, P);
        else PK<float>::particle_sums(s, view<float>(sp), sp.m, sp.w, ctx->partials, P);
        CK(cudaMemcpyAsync(h.data(), ctx->partials, sizeof(double) * 4 * P, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        for (int q = 0; q < 4; ++q) {
            double acc = 0;
            for (int b = 0; b < P; ++b) acc += h[q * P + b];
            out[q == 0 ? 0 : q + 2] += acc;
        }
    }
    const void* F[2];
    if (is_buneman(ctx)) { F[0] = ctx->E; F[1] = ctx->B; } else { F[0] = ctx->Ei; F[1] = ctx->Bi; }
    for (int f = 0; f < 2; ++f) {
        const int P = red_blocks(L);
        if (!is_buneman(ctx) || ctx->preal) PK<double>::field_sq_partials(s, F[f], L, ctx->partials, P);
        else PK<float>::field_sq_partials(s, F[f], L, ctx->partials, P);
        CK(cudaMemcpyAsync(h.data(), ctx->partials, sizeof(double) * P, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        double acc = 0;
        for (int b = 0; b < P; ++b) acc += h[b];
        out[1 + f] = acc * vol / (8 * pi);
    }
    return sync(ctx, "energy");
}

pic_status pic_profile(pic_ctx* ctx, int enable, double* phase_ms, long* launches) {
    if (!ctx) return PIC_ERR_ARG;
    prof_fold(ctx);
    if (phase_ms)
        for (int q = 0; q < PIC_PHASE_COUNT; ++q) phase_ms[q] = ctx->prof_ms[q];
    if (launches) *launches = ctx->launches;
    if (enable && !ctx->prof_on) {
        for (int q = 0; q < PIC_PHASE_COUNT; ++q) ctx->prof_ms[q] = 0;
        ctx->launches = 0;
    }
    ctx->prof_on = enable != 0;
    return sync(ctx, "profile");
}

// ---------------------------------------------------------------- checkpoint
namespace {

constexpr char kCkptMagic[8] = {'P', 'I', 'C', 'G', 'B', '3', '0', '0'};
constexpr int32_t kCkptVersion = 2;

struct CkptHeader {
    char magic[8];
    int32_t version, solver, particle_real, field_real, nx, ny, nz, nspecies, has_net, sorted, pad;
    int64_t step;
    double dx, dy, dz, dt, theta, eta, cfix;
};

// Device bytes to the file through a host buffer.
pic_status dev_write(pic_ctx* ctx, FILE* f, const void* d, size_t bytes, std::vector<char>& buf) {
    if (bytes == 0) return PIC_OK;
    buf.resize(bytes);
    CK(cudaMemcpyAsync(buf.data(), d, bytes, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    if (fwrite(buf.data(), 1, bytes, f) != bytes) return fail(ctx, PIC_ERR_ARG, "checkpoint write failed");
    return PIC_OK;
}

pic_status dev_read(pic_ctx* ctx, FILE* f, void* d, size_t bytes, std::vector<char>& buf) {
    if (bytes == 0) return PIC_OK;
    buf.resize(bytes);
    if (fread(buf.data(), 1, bytes, f) != bytes) return fail(ctx, PIC_ERR_ARG, "checkpoint truncated");
    CK(cudaMemcpyAsync(d, buf.data(), bytes, cudaMemcpyHostToDevice, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return PIC_OK;
}

struct FileCloser {
    FILE* f;
    ~FileCloser() { if (f) fclose(f); }
};

}  // namespace

pic_status pic_save_checkpoint(pic_ctx* ctx, const char* path) {
    if (!ctx || !path) return PIC_ERR_ARG;
    if (pic_status st0 = settle(ctx)) return st0;
    FILE* f = fopen(path, "wb");
    if (!f) return fail(ctx, PIC_ERR_ARG, std::string("cannot open ") + path);
    FileCloser fc{f};
    CkptHeader h{};
    memcpy(h.magic, kCkptMagic, 8);
    h.version = kCkptVersion;
    h.solver = ctx->cfg.solver; h.particle_real = ctx->cfg.particle_real; h.field_real = ctx->cfg.field_real;
    h.nx = ctx->g.nx; h.ny = ctx->g.ny; h.nz = ctx->g.nz;
    h.nspecies = (int32_t)ctx->sp.size();
    h.has_net = ctx->net && ctx->net->ready() ? 1 : 0;
    h.sorted = all_sorted(ctx) ? 1 : 0;
    h.step = ctx->step;
    h.dx = ctx->g.dx; h.dy = ctx->g.dy; h.dz = ctx->g.dz; h.dt = ctx->g.dt;
    h.theta = ctx->g.theta; h.eta = ctx->g.eta; h.cfix = ctx->g.cfix;
    if (fwrite(&h, sizeof(h), 1, f) != 1) return fail(ctx, PIC_ERR_ARG, "checkpoint write failed");
    std::vector<char> buf;
    pic_status st;
    for (auto& sp : ctx->sp) {
        const double qmw[3] = {sp.q, sp.m, sp.w};
        const int64_t n = sp.n;
        if (fwrite(qmw, sizeof(qmw), 1, f) != 1 || fwrite(&n, sizeof(n), 1, f) != 1)
            return fail(ctx, PIC_ERR_ARG, "checkpoint write failed");
        if ((st = dev_write(ctx, f, sp.cell, sizeof(int) * n, buf)) != PIC_OK) return st;
        if ((st = dev_write(ctx, f, sp.id, sizeof(int) * n, buf)) != PIC_OK) return st;
        for (int a = 0; a < 6; ++a)
            if ((st = dev_write(ctx, f, sp.a[a], ctx->rsz * n, buf)) != PIC_OK) return st;
        // tile offsets of the last sort (particles may have drifted since)
        if (h.sorted && (st = dev_write(ctx, f, sp.off, sizeof(int) * ((size_t)ctx->nkeys + 1), buf)) != PIC_OK)
            return st;
    }
    const size_t L = 3 * (size_t)ctx->g.N;
    if (is_buneman(ctx)) {
        const size_t fb = ctx->preal ? sizeof(double) : sizeof(float);
        if ((st = dev_write(ctx, f, ctx->E, fb * L, buf)) != PIC_OK) return st;
        if ((st = dev_write(ctx, f, ctx->B, fb * L, buf)) != PIC_OK) return st;
        if ((st = dev_write(ctx, f, ctx->J, sizeof(double) * L, buf)) != PIC_OK) return st;
    } else {
        if ((st = dev_write(ctx, f, ctx->Ei, sizeof(double) * L, buf)) != PIC_OK) return st;
        if ((st = dev_write(ctx, f, ctx->Bi, sizeof(double) * L, buf)) != PIC_OK) return st;
        if ((st = dev_write(ctx, f, ctx->Jh, sizeof(double) * L, buf)) != PIC_OK) return st;
    }
    if (h.has_net) {
        std::vector<float> p((size_t)Net::param_count());
        if ((st = ctx->net->get_params(ctx->s, p.data(), &ctx->err)) != PIC_OK) return st;
        if (fwrite(p.data(), sizeof(float), p.size(), f) != p.size()) return fail(ctx, PIC_ERR_ARG, "checkpoint write failed");
    }
    return PIC_OK;
}

pic_status pic_load_checkpoint(pic_ctx* ctx, const char* path) {
    if (!ctx || !path) return PIC_ERR_ARG;
    FILE* f = fopen(path, "rb");
    if (!f) return fail(ctx, PIC_ERR_ARG, std::string("cannot open ") + path);
    FileCloser fc{f};
    CkptHeader h{};
    if (fread(&h, sizeof(h), 1, f) != 1 || memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != kCkptVersion)
        return fail(ctx, PIC_ERR_ARG, "not a picpp_gb300 checkpoint");
    if (h.solver != ctx->cfg.solver || h.particle_real != ctx->cfg.particle_real ||
        h.field_real != ctx->cfg.field_real || h.nx != ctx->g.nx || h.ny != ctx->g.ny || h.nz != ctx->g.nz ||
        h.dx != ctx->g.dx || h.dy != ctx->g.dy || h.dz != ctx->g.dz || h.dt != ctx->g.dt ||
        h.theta != ctx->g.theta || h.eta != ctx->g.eta || h.cfix != ctx->g.cfix)
        return fail(ctx, PIC_ERR_ARG, "checkpoint configuration differs from the context's");
    if (h.nspecies > ctx->cfg.max_species) return fail(ctx, PIC_ERR_ARG, "too many species in the checkpoint");
    std::vector<char> buf;
    pic_status st;
    for (int q = 0; q < h.nspecies; ++q) {
        double qmw[3];
        int64_t n = 0;
        if (fread(qmw, sizeof(qmw), 1, f) != 1 || fread(&n, sizeof(n), 1, f) != 1 || n < 0)
            return fail(ctx, PIC_ERR_ARG, "checkpoint truncated");
        if (q >= (int)ctx->sp.size()) {
            if ((st = pic_add_species(ctx, qmw[0], qmw[1], qmw[2], (long)n, nullptr)) != PIC_OK) return st;
        }
        Species& sp = ctx->sp[q];
        if (n > sp.cap) return fail(ctx, PIC_ERR_NOMEM, "checkpoint species exceeds the capacity");
        sp.q = qmw[0]; sp.m = qmw[1]; sp.w = qmw[2];
        if ((st = dev_read(ctx, f, sp.cell, sizeof(int) * n, buf)) != PIC_OK) return st;
        if ((st = dev_read(ctx, f, sp.id, sizeof(int) * n, buf)) != PIC_OK) return st;
        for (int a = 0; a < 6; ++a)
            if ((st = dev_read(ctx, f, sp.a[a], ctx->rsz * n, buf)) != PIC_OK) return st;
        if (h.sorted && (st = dev_read(ctx, f, sp.off, sizeof(int) * ((size_t)ctx->nkeys + 1), buf)) != PIC_OK)
            return st;
        sp.n = n;
        sp.sorted = h.sorted != 0;
    }
    const size_t L = 3 * (size_t)ctx->g.N;
    if (is_buneman(ctx)) {
        const size_t fb = ctx->preal ? sizeof(double) : sizeof(float);
        if ((st = dev_read(ctx, f, ctx->E, fb * L, buf)) != PIC_OK) return st;
        if ((st = dev_read(ctx, f, ctx->B, fb * L, buf)) != PIC_OK) return st;
        if ((st = dev_read(ctx, f, ctx->J, sizeof(double) * L, buf)) != PIC_OK) return st;
    } else {
        if ((st = dev_read(ctx, f, ctx->Ei, sizeof(double) * L, buf)) != PIC_OK) return st;
        if ((st = dev_read(ctx, f, ctx->Bi, sizeof(double) * L, buf)) != PIC_OK) return st;
        if ((st = dev_read(ctx, f, ctx->Jh, sizeof(double) * L, buf)) != PIC_OK) return st;
    }
    if (h.has_net) {
        std::vector<float> p((size_t)Net::param_count());
        if (fread(p.data(), sizeof(float), p.size(), f) != p.size()) return fail(ctx, PIC_ERR_ARG, "checkpoint truncated");
        if (!ctx->net) ctx->net = new Net();
        if ((st = ctx->net->set_params(ctx->s, p.data(), &ctx->err)) != PIC_OK) return st;
    }
    ctx->step = h.step;
    ctx->moments_ready = ctx->efield_ready = ctx->mu_valid = false;
    ctx->fresh_sort = false;
    return sync(ctx, "load checkpoint");
}

// ---------------------------------------------------------------- density diagnostics
pic_status pic_update_density_parameters(pic_ctx* ctx) {
    if (!ctx) return PIC_ERR_ARG;
    if (pic_status st0 = settle(ctx)) return st0;
    const long long N = ctx->g.N;
    const int ns = (int)ctx->sp.size();
    cudaStream_t s = ctx->s;
    if (ctx->dens_ns < ns || !ctx->dens) {
        cudaFree(ctx->dens);
        ctx->dens = nullptr;
        ctx->dens_ns = 0;
        CK(dalloc(&ctx->dens, sizeof(double) * 5 * (size_t)N * (size_t)(ns > 0 ? ns : 1)));
        ctx->dens_ns = ns;
    }
    if (!ctx->dens_rho) CK(dalloc(&ctx->dens_rho, sizeof(double) * (size_t)N));
    CK(cudaMemsetAsync(ctx->dens, 0, sizeof(double) * 5 * (size_t)N * (size_t)ns, s));
    CK(cudaMemsetAsync(ctx->dens_rho, 0, sizeof(double) * (size_t)N, s));
    for (int q = 0; q < ns; ++q) {
        Species& sp = ctx->sp[q];
        double* base = ctx->dens + 5 * N * q;
        if (ctx->preal) PK<double>::density_deposit(s, ctx->g, view<double>(sp), sp.m, sp.w, base, base + N, base + 2 * N);
        else PK<float>::density_deposit(s, ctx->g, view<float>(sp), sp.m, sp.w, base, base + N, base + 2 * N);
        if (ctx->g.wall) launch_density_wall_fold(s, ctx->g, base, base + N, base + 2 * N);
        launch_density_finish(s, N, sp.q, base, base + N, base + 2 * N, ctx->dens_rho);
    }
    return sync(ctx, "density parameters");
}

pic_status pic_download_density(pic_ctx* ctx, int species, double* conc, double* energy, double* vel, double* rho) {
    if (!ctx) return PIC_ERR_ARG;
    pic_status st = check_species(ctx, species);
    if (st != PIC_OK) return st;
    if (!ctx->dens || species >= ctx->dens_ns) return fail(ctx, PIC_ERR_STATE, "update the density parameters first");
    const long long N = ctx->g.N;
    const double* base = ctx->dens + 5 * N * species;
    cudaStream_t s = ctx->s;
    if (conc) CK(cudaMemcpyAsync(conc, base, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    if (energy) CK(cudaMemcpyAsync(energy, base + N, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    if (vel) CK(cudaMemcpyAsync(vel, base + 2 * N, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s));
    if (rho) CK(cudaMemcpyAsync(rho, ctx->dens_rho, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    return sync(ctx, "download density");
}

// ---------------------------------------------------------------- learned preconditioner
long pic_nn_param_count(void) { return (long)Net::param_count(); }

static pic_status net_of(pic_ctx* ctx, bool need_ready) {
    if (!ctx) return PIC_ERR_ARG;
    if (is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not an implicit run");
    if (!ctx->net) ctx->net = new Net();
    if (need_ready && !ctx->net->ready())
        return fail(ctx, PIC_ERR_STATE, "learned preconditioner not initialised (pic_nn_init / pic_nn_set_params)");
    return PIC_OK;
}

pic_status pic_nn_init(pic_ctx* ctx, unsigned long long seed) {
    pic_status st = net_of(ctx, false);
    if (st != PIC_OK) return st;
    st = ctx->net->init(ctx->s, seed, &ctx->err);
    if (st != PIC_OK) return st;
    return sync(ctx, "nn init");
}

pic_status pic_nn_set_params(pic_ctx* ctx, const float* params) {
    if (!params) return PIC_ERR_ARG;
    pic_status st = net_of(ctx, false);
    if (st != PIC_OK) return st;
    return ctx->net->set_params(ctx->s, params, &ctx->err);
}

pic_status pic_nn_get_params(pic_ctx* ctx, float* params) {
    if (!params) return PIC_ERR_ARG;
    pic_status st = net_of(ctx, true);
    if (st != PIC_OK) return st;
    return ctx->net->get_params(ctx->s, params, &ctx->err);
}

pic_status pic_nn_train(pic_ctx* ctx, const pic_train_opts* opts, pic_train_info* info) {
    if (!opts) return PIC_ERR_ARG;
    pic_status st = net_of(ctx, true);
    if (st != PIC_OK) return st;
    if (!ctx->mu_valid && opts->source != 1)
        return fail(ctx, PIC_ERR_STATE, "no operator: update the electromagnetic parameters first");
    if (ctx->g.wall) return fail(ctx, PIC_ERR_STATE, "train on a periodic box (the network is convolutional)");
    if (opts->source == 1)
        st = ctx->net->train_triples(ctx->s, ctx->g, ctx->trip, *opts, info, ctx->partials, &ctx->err);
    else
        st = ctx->net->train(ctx->s, ctx->g, ctx->mu, *opts, info, ctx->partials, &ctx->err);
    if (st != PIC_OK) return st;
    return sync(ctx, "nn train");
}

pic_status pic_nn_wait_limit(pic_ctx* ctx, unsigned polls) {
    pic_status st = net_of(ctx, true);
    if (st != PIC_OK) return st;
    ctx->net->set_wait_limit(polls);
    return PIC_OK;
}

pic_status pic_nn_record(pic_ctx* ctx, int capacity) {
    if (!ctx || capacity < 0) return PIC_ERR_ARG;
    if (is_buneman(ctx)) return fail(ctx, PIC_ERR_STATE, "not an implicit run");
    if (capacity == 0) {
        ctx->trip.release();
        return PIC_OK;
    }
    pic_status st = ctx->trip.reserve(capacity, ctx->g.N, &ctx->err);
    if (st != PIC_OK) return st == PIC_ERR_CUDA ? fail(ctx, PIC_ERR_NOMEM, "no room for the triples") : st;
    return PIC_OK;
}

pic_status pic_nn_record_count(pic_ctx* ctx, int* count) {
    if (!ctx || !count) return PIC_ERR_ARG;
    *count = ctx->trip.count;
    return PIC_OK;
}

pic_status pic_nn_forward(pic_ctx* ctx, int n, int d, int h, int w, const float* x0, float* out) {
    if (!x0 || !out) return PIC_ERR_ARG;
    pic_status st = net_of(ctx, true);
    if (st != PIC_OK) return st;
    return ctx->net->forward_host(ctx->s, n, d, h, w, x0, out, &ctx->err);
}

pic_status pic_nn_loss_grad(pic_ctx* ctx, int n, int d, int h, int w, const float* x0, const float* target,
                            double* loss, float* grad) {
    if (!x0 || !target || !loss || !grad) return PIC_ERR_ARG;
    pic_status st = net_of(ctx, true);
    if (st != PIC_OK) return st;
    return ctx->net->loss_grad_host(ctx->s, n, d, h, w, x0, target, loss, grad, &ctx->err);
}

}  // extern "C"
