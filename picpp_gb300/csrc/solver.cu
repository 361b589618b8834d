// solver.cu -- GMRES drivers for the implicit Maxwell system A(mu) E = rhs.
//
// Vectors (3N unknowns, FP64) live on the device; Arnoldi scalars are
// computed on the device and read back once per iteration for the small
// Hessenberg/Givens algebra, which runs on the host in FP64.
#include <algorithm>
#include <cmath>
#include <vector>

#include "nn.hpp"
#include "solver.hpp"

namespace pic {

OpCoef make_opcoef(const GridP& g) {
    OpCoef oc{};
    const double d[3] = {g.dx, g.dy, g.dz};
    const int n[3] = {g.nx, g.ny, g.nz};
    oc.K = (g.theta * g.dt) * (g.theta * g.dt) * (g.cfix * g.cfix);
    for (int a = 0; a < 3; ++a) {
        oc.has[a] = n[a] > 1;
        oc.kd2[a] = oc.K / (d[a] * d[a]);
        for (int b = 0; b < 3; ++b) oc.kx4[a][b] = oc.K / (4 * d[a] * d[b]);
    }
    return oc;
}

void krylov_free(Krylov& k) {
    cudaFree(k.V); cudaFree(k.Z); cudaFree(k.w); cudaFree(k.mx); cudaFree(k.r); cudaFree(k.hdev); cudaFree(k.ydev);
    cudaFree(k.part); cudaFree(k.scal);
    cudaFree(k.mu32); cudaFree(k.V32); cudaFree(k.w32); cudaFree(k.mx32); cudaFree(k.h32); cudaFree(k.part32);
    cudaFree(k.cnt32);
    k = Krylov{};
}

namespace {

pic_status err(SolveCtx& c, pic_status st, const std::string& m) {
    if (c.err) *c.err = m;
    return st;
}

pic_status cerr(SolveCtx& c, cudaError_t e, const char* where) {
    return err(c, PIC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CKS(expr)                                              \
    do {                                                       \
        cudaError_t e_ = (expr);                               \
        if (e_ != cudaSuccess) return cerr(c, e_, #expr);      \
    } while (0)

pic_status ensure(SolveCtx& c, int cap, long long L) {
    Krylov& k = *c.k;
    if (k.cap >= cap && k.L == L) return PIC_OK;
    krylov_free(k);
    CKS(cudaMalloc(&k.V, sizeof(double) * (size_t)cap * L));
    CKS(cudaMalloc(&k.w, sizeof(double) * (size_t)L));
    CKS(cudaMalloc(&k.mx, sizeof(double) * (size_t)L));
    CKS(cudaMalloc(&k.r, sizeof(double) * (size_t)L));
    CKS(cudaMalloc(&k.hdev, sizeof(double) * 2 * (size_t)(cap + 2)));
    CKS(cudaMalloc(&k.ydev, sizeof(double) * (size_t)(cap + 2)));
    CKS(cudaMalloc(&k.part, sizeof(double) * (size_t)(cap + 2) * 1024));
    CKS(cudaMalloc(&k.scal, sizeof(double) * 16));
    k.cap = cap;
    k.L = L;
    return PIC_OK;
}

double read1(SolveCtx& c, const double* d, pic_status* st) {
    double h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, c.s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.s);
    if (e != cudaSuccess) *st = cerr(c, e, "read scalar");
    return h;
}

pic_status check_finite(SolveCtx& c, const double* a, long long n) {
    CKS(cudaMemsetAsync(c.flag, 0, sizeof(int), c.s));
    launch_nonfinite(c.s, a, n, c.flag);
    int bad = 0;
    CKS(cudaMemcpyAsync(&bad, c.flag, sizeof(int), cudaMemcpyDeviceToHost, c.s));
    CKS(cudaStreamSynchronize(c.s));
    if (bad) return err(c, PIC_ERR_NUMERIC, "non-finite value in the Maxwell system");
    return PIC_OK;
}

// generalizedMinimalResidualMethod (PIC++/specialmath.cpp:367-671) semantics.
pic_status gmres_reference(SolveCtx& c, const OpCoef& oc, const double* rhs, double* x, const pic_solve_opts& o,
                           pic_solve_info* info) {
    const GridP& g = *c.g;
    const long long L = 3 * g.N;
    const int P = red_blocks(L);
    const int maxIter = o.max_iter > 0 ? o.max_iter : 50;
    pic_status st = PIC_OK;
    if ((st = ensure(c, maxIter + 2, L)) != PIC_OK) return st;
    Krylov& k = *c.k;
    launch_dot(c.s, rhs, rhs, L, k.part, P, k.scal, 1);
    double norm = read1(c, k.scal, &st);
    if (st != PIC_OK) return st;
    if (norm == 0) {
        CKS(cudaMemsetAsync(x, 0, sizeof(double) * L, c.s));
        if (info) { info->iterations = 0; info->rel_residual = 0; }
        return PIC_OK;
    }
    auto Vp = [&](int m) { return k.V + (long long)m * L; };
    launch_div(c.s, Vp(0), rhs, norm, L);
    launch_dot(c.s, Vp(0), Vp(0), L, k.part, P, k.scal, 1);
    const double normR = read1(c, k.scal, &st);
    if (st != PIC_OK) return st;
    // matrixDimension of the reference: 3 x its cells (the physical ones of a wall box)
    const long long dim = g.wall ? 3LL * (g.nx - 2) * g.ny * g.nz : L;
    double tolRel = o.tol / (double)dim;
    if (tolRel < 1e-15) tolRel = 1e-15;
    const int cap = maxIter + 2;
    std::vector<double> H((size_t)cap * cap, 0.0), Q((size_t)cap * cap, 0.0), Qo((size_t)cap * cap, 0.0),
        R((size_t)cap * cap, 0.0), y(cap, 0.0), hcol(cap, 0.0);
    auto M = [&](std::vector<double>& A, int i, int j) -> double& { return A[(size_t)i * cap + j]; };
    int n = 2;
    const double beta = 1.0;
    double relErr = 1.0;
    const long long lim = std::min<long long>(maxIter, dim + 3);
    while (relErr > tolRel && n < lim) {
        launch_maxwell_apply(c.s, g, oc, c.mu, Vp(n - 2), Vp(n - 1), k.mx);
        for (int m = 0; m < n - 1; ++m) {
            launch_dot(c.s, Vp(m), Vp(n - 1), L, k.part, P,k.hdev + m, 0);
            launch_axpy_minus_dev(c.s, Vp(n - 1), Vp(m), k.hdev + m, L);
        }
        launch_dot(c.s, Vp(n - 1), Vp(n - 1), L, k.part, P,k.hdev + (n - 1), 1);
        launch_scale_inv_dev(c.s, Vp(n - 1), Vp(n - 1), k.hdev + (n - 1), L);
        CKS(cudaMemcpyAsync(hcol.data(), k.hdev, sizeof(double) * n, cudaMemcpyDeviceToHost, c.s));
        CKS(cudaStreamSynchronize(c.s));
        for (int m = 0; m < n; ++m) M(H, m, n - 2) = hcol[m];
        if (n == 2) {
            double rho = M(H, 0, 0), sigma = M(H, 1, 0);
            double mod = std::sqrt(rho * rho + sigma * sigma);
            double cs = rho / mod, sn = sigma / mod;
            M(Q, 0, 0) = cs; M(Q, 0, 1) = sn; M(Q, 1, 0) = -sn; M(Q, 1, 1) = cs;
            M(R, 0, 0) = mod; M(R, 1, 0) = 0;
        } else {
            Qo = Q;
            for (int j = 0; j < n - 2; ++j) M(R, n - 1, j) = 0;
            for (int i = 0; i < n - 1; ++i) M(Q, i, n - 1) = 0;
            for (int j = 0; j < n - 1; ++j) M(Q, n - 1, j) = 0;
            M(Q, n - 1, n - 1) = 1;
            for (int i = 0; i < n; ++i) {
                double sum = 0;
                for (int j = 0; j < n; ++j) sum += M(Q, i, j) * M(H, j, n - 2);
                M(R, i, n - 2) = sum;
            }
            double rho = M(R, n - 2, n - 2), sigma = M(R, n - 1, n - 2);
            double mod = std::sqrt(rho * rho + sigma * sigma);
            double cs = rho / mod, sn = sigma / mod;
            M(R, n - 2, n - 2) = mod; M(R, n - 1, n - 2) = 0;
            for (int j = 0; j < n - 1; ++j) {
                M(Q, n - 2, j) = cs * M(Qo, n - 2, j);
                M(Q, n - 1, j) = -sn * M(Qo, n - 2, j);
            }
            M(Q, n - 2, n - 1) = sn; M(Q, n - 1, n - 1) = cs;
        }
        for (int i = n - 2; i >= 0; --i) {
            y[i] = beta * M(Q, i, 0);
            for (int j = n - 2; j > i; --j) y[i] -= M(R, i, j) * y[j];
            if (M(R, i, i) > 0) y[i] /= M(R, i, i); else y[i] = 0;
        }
        relErr = std::fabs(beta * M(Q, n - 1, 0)) / normR;
        n++;
    }
    n = n - 1;
    CKS(cudaMemcpyAsync(k.ydev, y.data(), sizeof(double) * std::max(n - 1, 1), cudaMemcpyHostToDevice, c.s));
    launch_combine(c.s, x, k.V, L, n - 1, k.ydev, norm, 0, L);
    if (info) {
        info->iterations = n - 1;
        info->restarts = 0;
        info->rel_residual = relErr;
    }
    CKS(cudaStreamSynchronize(c.s));
    return PIC_OK;
}

pic_status ensure_z(SolveCtx& c, int m, long long L) {
    Krylov& k = *c.k;
    if (k.zcap >= m && k.Z) return PIC_OK;
    cudaFree(k.Z);
    k.Z = nullptr;
    k.zcap = 0;
    CKS(cudaMalloc(&k.Z, sizeof(double) * (size_t)m * L));
    k.zcap = m;
    return PIC_OK;
}

// ---- mixed-precision right preconditioner: z = an FP32 GMRES solve of
// A z = v from zero, at most S Arnoldi steps, stopped once its residual
// estimate falls to tol |v|.  FP64 runs at about 1/64 of the FP32 rate on
// this GPU, so the bulk of the Krylov work (operator applies, Gram-Schmidt)
// moves to FP32, where it is bound by memory traffic; the outer flexible
// GMRES keeps FP64 vectors and checks the FP64 true residual, so the solve
// reaches the same tolerance.  One classical Gram-Schmidt pass per step
// (the inner solve only preconditions: lost orthogonality costs it
// accuracy, not the outer solve correctness).  The Givens rotations and the
// back-substitution run on the device (one thread each), so an apply needs
// no host round trip; after the stop every remaining inner kernel returns
// at entry (the done flag), which leaves only their launches.
pic_status ensure_inner(SolveCtx& c, int S, long long L) {
    Krylov& k = *c.k;
    if (k.steps32 >= S && k.V32) return PIC_OK;
    cudaFree(k.mu32); cudaFree(k.V32); cudaFree(k.w32); cudaFree(k.mx32); cudaFree(k.h32); cudaFree(k.part32);
    cudaFree(k.cnt32);
    k.mu32 = nullptr; k.V32 = nullptr; k.w32 = nullptr; k.mx32 = nullptr; k.h32 = nullptr; k.part32 = nullptr;
    k.cnt32 = nullptr;
    k.steps32 = 0;
    CKS(cudaMalloc(&k.mu32, sizeof(float) * 3 * (size_t)L));
    CKS(cudaMalloc(&k.V32, sizeof(float) * (size_t)(S + 1) * L));
    CKS(cudaMalloc(&k.w32, sizeof(float) * (size_t)L));
    CKS(cudaMalloc(&k.mx32, sizeof(float) * (size_t)L));
    CKS(cudaMalloc(&k.h32, sizeof(double) * (size_t)InnerLayout{S}.size()));
    CKS(cudaMalloc(&k.part32, sizeof(double) * (size_t)(S + 2) * 1024));
    CKS(cudaMalloc(&k.cnt32, sizeof(unsigned) * 4));   // [0] reduction counter, [1] done, [2] columns
    CKS(cudaMemsetAsync(k.cnt32, 0, sizeof(unsigned) * 4, c.s));
    k.steps32 = S;
    return PIC_OK;
}

pic_status inner_apply(SolveCtx& c, const OpCoef& oc, int S, double tol, const double* v, double* z) {
    const GridP& g = *c.g;
    Krylov& k = *c.k;
    const long long L = 3 * g.N;
    const int P = red_blocks(L);
    const InnerLayout lay{S};
    auto V = [&](int j) { return k.V32 + (long long)j * L; };
    double* h = k.h32;
    unsigned* cnt = k.cnt32;
    unsigned* done = k.cnt32 + 1;
    launch_to_f32(c.s, k.w32, v, L);
    launch_dot_f32(c.s, k.w32, k.w32, L, k.part32, P, h, cnt);
    launch_normalize_f32(c.s, V(0), k.w32, h, L, done);
    for (int j = 0; j < S; ++j) {
        float* w = V(j + 1);
        double* col = h + lay.h() + (long long)j * (S + 1);
        launch_maxwell_apply_f32(c.s, g, oc, k.mu32, V(j), w, k.mx32, done);
        launch_multi_dot_f32(c.s, k.V32, L, j + 1, w, L, k.part32, P, col, cnt, done);
        launch_axpy_norm_f32(c.s, w, k.V32, L, j + 1, col, L, k.part32, P, h + lay.hn() + j, cnt, done);
        launch_normalize_f32(c.s, w, w, h + lay.hn() + j, L, done);
        launch_inner_givens(c.s, j, S, h, tol, k.cnt32);
    }
    launch_inner_backsolve(c.s, S, h, k.cnt32);
    launch_combine_f32(c.s, z, k.V32, L, k.cnt32 + 2, h + lay.y(), 1.0, L);
    CKS(cudaGetLastError());
    return PIC_OK;
}

// Restarted GMRES(m): classical Gram-Schmidt with a second pass where the
// first one cancels, Givens rotations on the host (one stream
// synchronisation per iteration, two with the second pass), FP64 true
// residual at every restart.  With
// a network (pc != nullptr) it is flexible GMRES (Saad 1993) with the right
// preconditioner z_j = pc(v_j), x += Z y; a cycle that does not halve the
// true residual, or a non-finite preconditioned direction, switches the
// rest of the solve to plain GMRES from the current iterate.  With inner > 0
// the right preconditioner is instead the FP32 inner solve of inner steps.
pic_status gmres_restarted(SolveCtx& c, const OpCoef& oc, const double* b, double* x, const pic_solve_opts& o,
                           pic_solve_info* info, Net* pc = nullptr, int inner = 0) {
    const GridP& g = *c.g;
    Net* const net = pc;   // pc becomes nullptr on a fallback
    bool have = pc != nullptr || inner > 0;   // a right preconditioner is in use
    const long long L = 3 * g.N;
    const int P = red_blocks(L);
    const int m = std::max(1, o.restart > 0 ? o.restart : 30);
    const int maxIter = o.max_iter > 0 ? o.max_iter : 1000;
    const double tol = o.tol > 0 ? o.tol : 1e-8;
    pic_status st = PIC_OK;
    if ((st = ensure(c, m + 1, L)) != PIC_OK) return st;
    if (have && (st = ensure_z(c, m, L)) != PIC_OK) return st;
    if (inner > 0 && (st = ensure_inner(c, inner, L)) != PIC_OK) return st;
    Krylov& k = *c.k;
    if (inner > 0) launch_to_f32(c.s, k.mu32, c.mu, 3 * L);   // mu for the FP32 operator
    auto Vp = [&](int j) { return k.V + (long long)j * L; };
    auto Zp = [&](int j) { return k.Z + (long long)j * L; };
    bool fallback = false;
    double prev_rel = 1.0;
    launch_dot(c.s, b, b, L, k.part, P,k.scal, 1);
    const double bnorm = read1(c, k.scal, &st);
    if (st != PIC_OK) return st;
    CKS(cudaMemsetAsync(x, 0, sizeof(double) * L, c.s));
    if (bnorm == 0) {
        if (info) { info->iterations = 0; info->restarts = 0; info->rel_residual = 0; }
        return PIC_OK;
    }
    CKS(cudaMemcpyAsync(k.r, b, sizeof(double) * L, cudaMemcpyDeviceToDevice, c.s));
    std::vector<double> H((size_t)(m + 1) * m, 0.0), gv(m + 1), cs(m), sn(m), h1(m + 2), h2(m + 2), y(m);
    auto Hm = [&](int i, int j) -> double& { return H[(size_t)i * m + j]; };
    int total = 0, restarts = 0;
    double rel = 1.0;
    for (;;) {
        launch_dot(c.s, k.r, k.r, L, k.part, P,k.scal, 1);
        const double beta = read1(c, k.scal, &st);
        if (st != PIC_OK) return st;
        rel = beta / bnorm;
        if (!std::isfinite(rel)) return err(c, PIC_ERR_NUMERIC, "non-finite residual");
        if (rel <= tol || total >= maxIter) break;
        if (have && restarts > 0 && rel > 0.5 * prev_rel) { pc = nullptr; have = false; fallback = true; }
        prev_rel = rel;
        launch_scale(c.s, Vp(0), k.r, 1.0 / beta, L);   // one reciprocal, not an FP64 division per element
        std::fill(gv.begin(), gv.end(), 0.0);
        gv[0] = beta;
        int j = 0;
        bool bad = false, degenerate = false;
        for (; j < m; ++j) {
            double* w = Vp(j + 1);
            if (have) {
                if (pc) {
                    if ((st = pc->apply(c.s, g, c.mu, Vp(j), Zp(j), k.scal + 8, c.partials, c.err)) != PIC_OK) return st;
                } else {
                    // the inner solve only needs to bring this direction's
                    // share of the residual to the tolerance: a rough solve
                    // once the outer residual is small, FP32's limit early on
                    const double now = std::fabs(gv[j]) / bnorm;
                    const double itol = std::min(0.5, std::max(1e-7, 0.3 * tol / std::max(now, 1e-300)));
                    if ((st = inner_apply(c, oc, inner, itol, Vp(j), Zp(j))) != PIC_OK) return st;
                }
                launch_maxwell_apply(c.s, g, oc, c.mu, Zp(j), w, k.mx);
            } else {
                launch_maxwell_apply(c.s, g, oc, c.mu, Vp(j), w, k.mx);
            }
            // classical Gram-Schmidt; the second pass only when the first
            // left less than 1/sqrt(2) of |w| (Kahan's "twice is enough"
            // test): every pass is (j + 1) FP64 dot products and updates of
            // length L, arithmetic-bound on this GPU.  w is V[j + 1], so the
            // first multi-dot over j + 2 vectors also returns |w|^2.
            launch_multi_dot(c.s, k.V, L, j + 2, w, L, k.part, P, k.hdev);
            launch_multi_axpy_minus(c.s, w, k.V, L, j + 1, k.hdev, 1, L);
            launch_dot(c.s, w, w, L, k.part, P, k.scal + 2, 1);
            CKS(cudaMemcpyAsync(h1.data(), k.hdev, sizeof(double) * (j + 2), cudaMemcpyDeviceToHost, c.s));
            double after = 0;
            CKS(cudaMemcpyAsync(&after, k.scal + 2, sizeof(double), cudaMemcpyDeviceToHost, c.s));
            CKS(cudaStreamSynchronize(c.s));
            const double before = std::sqrt(std::max(h1[j + 1], 0.0));
            const bool second = !(after >= 0.7071067811865476 * before);
            if (second) {
                launch_multi_dot(c.s, k.V, L, j + 1, w, L, k.part, P, k.hdev + (m + 2));
                launch_multi_axpy_minus(c.s, w, k.V, L, j + 1, k.hdev + (m + 2), 1, L);
                launch_dot(c.s, w, w, L, k.part, P, k.hdev + (j + 1), 1);
                CKS(cudaMemcpyAsync(h2.data(), k.hdev + (m + 2), sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, c.s));
                CKS(cudaMemcpyAsync(&h1[j + 1], k.hdev + (j + 1), sizeof(double), cudaMemcpyDeviceToHost, c.s));
            } else {
                std::fill(h2.begin(), h2.begin() + (j + 1), 0.0);
                h1[j + 1] = after;
                CKS(cudaMemcpyAsync(k.hdev + (j + 1), k.scal + 2, sizeof(double), cudaMemcpyDeviceToDevice, c.s));
            }
            launch_scale_inv_dev(c.s, w, w, k.hdev + (j + 1), L);
            // only the second pass copies values back; otherwise the host's
            // Givens update overlaps the normalisation and the next apply
            if (second) CKS(cudaStreamSynchronize(c.s));
            if (have) {
                // a non-finite direction, or one already in the Krylov space
                // (|h_{j+1,j}| below 1e-10 |A z_j|), ends the cycle
                bool fin = std::isfinite(h1[j + 1]);
                double hn2 = h1[j + 1] * h1[j + 1];
                for (int i = 0; i <= j; ++i) {
                    fin = fin && std::isfinite(h1[i]) && std::isfinite(h2[i]);
                    hn2 += (h1[i] + h2[i]) * (h1[i] + h2[i]);
                }
                if (!fin) { bad = true; break; }
                if (!(h1[j + 1] > 1e-10 * std::sqrt(hn2))) { degenerate = true; break; }
            }
            for (int i = 0; i <= j; ++i) Hm(i, j) = h1[i] + h2[i];
            Hm(j + 1, j) = h1[j + 1];
            for (int i = 0; i < j; ++i) {
                double t = cs[i] * Hm(i, j) + sn[i] * Hm(i + 1, j);
                Hm(i + 1, j) = -sn[i] * Hm(i, j) + cs[i] * Hm(i + 1, j);
                Hm(i, j) = t;
            }
            double a = Hm(j, j), bb = Hm(j + 1, j);
            double mod = std::hypot(a, bb);
            if (mod == 0) { cs[j] = 1; sn[j] = 0; } else { cs[j] = a / mod; sn[j] = bb / mod; }
            Hm(j, j) = mod;
            Hm(j + 1, j) = 0;
            gv[j + 1] = -sn[j] * gv[j];
            gv[j] = cs[j] * gv[j];
            ++total;
            if (std::fabs(gv[j + 1]) / bnorm <= tol || total >= maxIter || h1[j + 1] == 0) { ++j; break; }
        }
        if (bad) {   // the preconditioner produced a non-finite direction: drop the cycle
            pc = nullptr;
            have = false;
            fallback = true;
            ++restarts;
            continue;
        }
        const int kk = std::min(j, m);
        for (int i = kk - 1; i >= 0; --i) {
            double s = gv[i];
            for (int q = i + 1; q < kk; ++q) s -= Hm(i, q) * y[q];
            y[i] = Hm(i, i) != 0 ? s / Hm(i, i) : 0.0;
        }
        CKS(cudaMemcpyAsync(k.ydev, y.data(), sizeof(double) * std::max(kk, 1), cudaMemcpyHostToDevice, c.s));
        if (have) {
            // keep x and r: a preconditioned cycle that raises the true
            // residual (rounding with nearly dependent directions) is undone
            CKS(cudaMemcpyAsync(Vp(0), x, sizeof(double) * L, cudaMemcpyDeviceToDevice, c.s));
            CKS(cudaMemcpyAsync(Vp(1), k.r, sizeof(double) * L, cudaMemcpyDeviceToDevice, c.s));
        }
        launch_combine(c.s, x, have ? k.Z : k.V, L, kk, k.ydev, 1.0, 1, L);
        launch_maxwell_apply(c.s, g, oc, c.mu, x, k.w, k.mx);
        launch_residual(c.s, k.r, b, k.w, L);
        ++restarts;
        if (have) {
            launch_dot(c.s, k.r, k.r, L, k.part, P, k.scal, 1);
            const double after = read1(c, k.scal, &st) / bnorm;
            if (st != PIC_OK) return st;
            if (!(after < rel)) {
                CKS(cudaMemcpyAsync(x, Vp(0), sizeof(double) * L, cudaMemcpyDeviceToDevice, c.s));
                CKS(cudaMemcpyAsync(k.r, Vp(1), sizeof(double) * L, cudaMemcpyDeviceToDevice, c.s));
                degenerate = true;
            }
            if (degenerate) { pc = nullptr; have = false; fallback = true; }
        }
    }
    if (net && (st = net->check_tc(c.s, c.err)) != PIC_OK) return st;
    if (info) {
        info->iterations = total;
        info->restarts = restarts;
        info->rel_residual = rel;
        info->used_fallback = fallback ? 1 : 0;
    }
    return rel <= tol ? PIC_OK : err(c, PIC_ERR_NOT_CONVERGED, "GMRES did not reach the tolerance");
}

}  // namespace

pic_status krylov_solve(SolveCtx& c, const double* rhs, double* x, const pic_solve_opts& o, pic_solve_info* info) {
    const long long L = 3 * c.g->N;
    pic_status st = check_finite(c, rhs, L);
    if (st != PIC_OK) return st;
    st = check_finite(c, c.mu, 3 * L);
    if (st != PIC_OK) return st;
    const OpCoef oc = make_opcoef(*c.g);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, c.s);
    if (info) *info = pic_solve_info{};
    switch (o.method) {
        case PIC_GMRES_REFERENCE: st = gmres_reference(c, oc, rhs, x, o, info); break;
        case PIC_GMRES_RESTARTED: st = gmres_restarted(c, oc, rhs, x, o, info); break;
        case PIC_FGMRES_LEARNED:
            if (!c.net || !c.net->ready()) {
                st = err(c, PIC_ERR_STATE, "learned preconditioner not initialised (pic_nn_init / pic_nn_set_params)");
            } else if (c.g->nx % 4 || c.g->ny % 4 || c.g->nz % 4) {
                st = err(c, PIC_ERR_ARG, "learned preconditioner needs box axes that are multiples of 4");
            } else {
                st = gmres_restarted(c, oc, rhs, x, o, info, c.net);
            }
            break;
        case PIC_FGMRES_MIXED:
            st = o.inner < 0 || o.inner > 64 ? err(c, PIC_ERR_ARG, "inner steps must lie in 0..64")
                                              : gmres_restarted(c, oc, rhs, x, o, info, nullptr, o.inner > 0 ? o.inner : 12);
            break;
        default: st = err(c, PIC_ERR_ARG, "unknown solver method"); break;
    }
    cudaEventRecord(e1, c.s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (info) info->seconds = ms * 1e-3;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
}

}  // namespace pic
