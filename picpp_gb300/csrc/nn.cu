// nn.cu -- host side of the learned preconditioner (nn.hpp): parameter
// vector, activation buffers, forward / backward / Adam, the FGMRES
// preconditioner apply and the training loop on the box's operator.
#include <cmath>
#include <cstring>

#include "kernels.hpp"
#include "nn.hpp"
#include "conv_tc.cuh"
#include "nn_kernels.cuh"
#include "solver.hpp"

namespace pic {

using nn::bf16;
using nn::Dims;

namespace {

#define NCK(expr)                                                                    \
    do {                                                                             \
        cudaError_t e_ = (expr);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            if (err) *err = std::string(#expr) + ": " + cudaGetErrorString(e_);      \
            return PIC_ERR_CUDA;                                                     \
        }                                                                            \
    } while (0)

std::vector<NetLayer> make_layers() {
    std::vector<NetLayer> L = {
        {"e0a", 16, 16, 0}, {"e0b", 16, 16, 0}, {"e1a", 16, 32, 0}, {"e1b", 32, 32, 0},
        {"e2a", 32, 64, 0}, {"e2b", 64, 64, 0}, {"d1a", 96, 32, 0}, {"d1b", 32, 32, 0},
        {"d0a", 48, 16, 0}, {"d0b", 16, 16, 0}, {"head", 16, 16, 0},
    };
    long long off = 0;
    for (auto& l : L) {
        l.woff = off;
        l.boff = off + 27LL * l.cin * l.cout;
        off = l.boff + l.cout;
    }
    return L;
}

enum { E0A, E0B, E1A, E1B, E2A, E2B, D1A, D1B, D0A, D0B, HEAD };

int gs(long long n) { return grid_for(n, 256, 16); }

template <int CI, int CO>
void conv_t(cudaStream_t s, const bf16* x, const bf16* W, const float* b, bf16* y16, float* y32, Dims d, int relu,
            int* err, unsigned wait_limit) {
    static bool attr = false;
    const size_t sm = nn::tc_conv_smem_bytes(CI, CO);
    if (!attr) {
        cudaFuncSetAttribute(nn::k_conv3_tc<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        attr = true;
    }
    dim3 grid((d.W + nn::kTcW - 1) / nn::kTcW, (d.H + nn::kTcH - 1) / nn::kTcH, d.N * d.D);
    nn::k_conv3_tc<CI, CO><<<grid, nn::kTcThreads, sm, s>>>(x, W, b, y16, y32, d.N, d.D, d.H, d.W, relu, err,
                                                              wait_limit);
}

// Every (cin, cout) pair of the forward layers and of their input-gradient
// (transposed) convolutions.
void conv(cudaStream_t s, int ci, int co, const bf16* x, const bf16* W, const float* b, bf16* y16, float* y32, Dims d,
          int relu, int* err, unsigned wait_limit) {
#define PIC_CONV(A, B) \
    if (ci == A && co == B) return conv_t<A, B>(s, x, W, b, y16, y32, d, relu, err, wait_limit)
    PIC_CONV(16, 16); PIC_CONV(16, 32); PIC_CONV(32, 16); PIC_CONV(32, 32); PIC_CONV(32, 64); PIC_CONV(64, 32);
    PIC_CONV(64, 64); PIC_CONV(96, 32); PIC_CONV(32, 96); PIC_CONV(48, 16); PIC_CONV(16, 48);
#undef PIC_CONV
}

template <int CI, int CO>
void wgrad_t(cudaStream_t s, const bf16* x, const bf16* g, Dims d, float* dW, float* db) {
    static bool attr = false;
    const size_t sm = (size_t)nn::kWgVox * (CI + CO) * sizeof(float);
    if (!attr) {
        cudaFuncSetAttribute(nn::k_wgrad<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        attr = true;
    }
    dim3 grid((unsigned)((d.vox() + nn::kWgVox - 1) / nn::kWgVox), 27);
    nn::k_wgrad<CI, CO><<<grid, 256, sm, s>>>(x, g, d, dW, db);
}

void wgrad(cudaStream_t s, int ci, int co, const bf16* x, const bf16* g, Dims d, float* dW, float* db) {
#define PIC_WG(A, B) \
    if (ci == A && co == B) return wgrad_t<A, B>(s, x, g, d, dW, db)
    PIC_WG(16, 16); PIC_WG(16, 32); PIC_WG(32, 32); PIC_WG(32, 64); PIC_WG(64, 64); PIC_WG(96, 32); PIC_WG(48, 16);
#undef PIC_WG
}

// ---- data movement between the Krylov vectors and the network ----------
// x0[v][16] = (r / s (3), mu_xx, mu_yy, mu_zz, 0 ...) for every cell v.
__global__ void k_pack_box(const double* __restrict__ r, double inv_s, const double* __restrict__ mu,
                           bf16* __restrict__ x0, long long N) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < N; v += (long long)gridDim.x * blockDim.x) {
        __align__(16) bf16 c[16];
        c[0] = __double2bfloat16(r[v] * inv_s);
        c[1] = __double2bfloat16(r[N + v] * inv_s);
        c[2] = __double2bfloat16(r[2 * N + v] * inv_s);
        c[3] = __double2bfloat16(mu[v]);
        c[4] = __double2bfloat16(mu[4 * N + v]);
        c[5] = __double2bfloat16(mu[8 * N + v]);
#pragma unroll
        for (int q = 6; q < 16; ++q) c[q] = __float2bfloat16(0.f);
        uint4* dst = reinterpret_cast<uint4*>(x0 + v * 16);
        dst[0] = reinterpret_cast<const uint4*>(c)[0];
        dst[1] = reinterpret_cast<const uint4*>(c)[1];
    }
}

// z[c][v] = g r[c][v] + s * out[v][c], c < 3: the gated identity plus the
// network's correction (g, a parameter, at *gate).
__global__ void k_unpack_box(const float* __restrict__ out, double s, const double* __restrict__ r,
                             const float* __restrict__ gate, double* __restrict__ z, long long N) {
    const double gg = (double)*gate;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < N; v += (long long)gridDim.x * blockDim.x) {
        const float* o = out + v * 16;
        z[v] = gg * r[v] + s * (double)o[0];
        z[N + v] = gg * r[N + v] + s * (double)o[1];
        z[2 * N + v] = gg * r[2 * N + v] + s * (double)o[2];
    }
}

// dL/dg = f * sum_q <A^T (A z_q - r_q), r_q> (the dot products in d[0..nb)).
__global__ void k_gate_grad(const double* __restrict__ d, int nb, double f, float* __restrict__ gg) {
    double t = 0;
    for (int q = 0; q < nb; ++q) t += d[q];
    *gg += (float)(f * t);
}

// a *= sqrt(n) / |a| (unit root-mean-square), |a| in norm[0].
__global__ void k_rescale_by_norm(double* __restrict__ a, long long n, const double* __restrict__ norm) {
    const double f = norm[0] > 0 ? sqrt((double)n) / norm[0] : 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        a[e] *= f;
}

// e = Az - r (in place in e); w * |e|^2 added to *loss.
__global__ void k_sub_loss(double* __restrict__ e, const double* __restrict__ r, long long n, double w,
                           double* __restrict__ loss) {
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double d = e[i] - r[i];
        e[i] = d;
        s += d * d;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(loss, w * s);
}

// g[v][c] = f * a[c][v] for c < 3, 0 for the padding channels (FP32).
__global__ void k_pack_grad(const double* __restrict__ a, double f, float* __restrict__ g, long long N) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < N; v += (long long)gridDim.x * blockDim.x) {
        float* o = g + v * 16;
        o[0] = (float)(f * a[v]);
        o[1] = (float)(f * a[N + v]);
        o[2] = (float)(f * a[2 * N + v]);
#pragma unroll
        for (int q = 3; q < 16; ++q) o[q] = 0.f;
    }
}

__device__ __forceinline__ unsigned long long nn_mix(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// White noise in [-1, 1) (splitmix64 of (seed, index)).
__global__ void k_noise(double* __restrict__ x, long long n, unsigned long long seed) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        x[e] = 2.0 * ((nn_mix(seed * 0x100000001B3ull + (unsigned long long)e) >> 11) * 0x1.0p-53) - 1.0;
}

__global__ void k_d2f(const double* __restrict__ a, float* __restrict__ b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

__global__ void k_f2d(const float* __restrict__ a, double* __restrict__ b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

// y = a y + b x
__global__ void k_axpby(double* __restrict__ y, const double* __restrict__ x, double a, double b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = a * y[i] + b * x[i];
}

// One periodic binomial (1 2 1) / 4 pass along every active axis of a
// 3-component field, src -> dst.
__global__ void k_smooth(GridP g, const double* __restrict__ src, double* __restrict__ dst) {
    const long long tot = 3 * g.N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
        const long long c = e / g.N, id = e % g.N;
        int i, j, k;
        decode(g, (int)id, i, j, k);
        const double* a = src + c * g.N;
        double s = 0.0, wsum = 0.0;
        for (int dk = -1; dk <= 1; ++dk) {
            if (!g.z3 && dk) continue;
            for (int dj = -1; dj <= 1; ++dj) {
                if (!g.y3 && dj) continue;
                for (int di = -1; di <= 1; ++di) {
                    if (g.nx == 1 && di) continue;
                    const double w = (di ? 1.0 : 2.0) * (dj ? 1.0 : 2.0) * (dk ? 1.0 : 2.0);
                    s += w * a[linw(g, i + di, j + dj, k + dk)];
                    wsum += w;
                }
            }
        }
        dst[e] = s / wsum;
    }
}

__global__ void k_f32_to_bf16(const float* __restrict__ a, bf16* __restrict__ b, long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        b[e] = __float2bfloat16(a[e]);
}

__global__ void k_he_init(float* __restrict__ p, long long n, int cin, int cout, int cin_real, int cout_real,
                          unsigned long long seed, float scale) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int ci = (int)(e % cin), co = (int)((e / cin) % cout);
        float val = 0.f;
        if (ci < cin_real && co < cout_real) {
            // Box-Muller on two splitmix64 uniforms
            const double u1 = ((nn_mix(seed * 0x9E37ull + 2 * (unsigned long long)e) >> 11) + 1) * 0x1.0p-53;
            const double u2 = (nn_mix(seed * 0x9E37ull + 2 * (unsigned long long)e + 1) >> 11) * 0x1.0p-53;
            val = (float)(sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2)) * scale;
        }
        p[e] = val;
    }
}

}  // namespace

// ---- buffers ------------------------------------------------------------
struct NetBuffers {
    Dims dm0{}, dm1{}, dm2{};
    bool grads = false;
    bf16 *x0 = nullptr, *e0a = nullptr, *e0 = nullptr, *p1 = nullptr, *e1a = nullptr, *e1 = nullptr, *p2 = nullptr;
    bf16 *e2a = nullptr, *e2 = nullptr, *c1 = nullptr, *d1a = nullptr, *d1 = nullptr, *c0 = nullptr, *d0a = nullptr;
    bf16 *d0 = nullptr, *g16 = nullptr;
    float* out = nullptr;
    float *A0 = nullptr, *B0 = nullptr, *S0 = nullptr, *A1 = nullptr, *B1 = nullptr, *S1 = nullptr, *A2 = nullptr,
          *B2 = nullptr;
    float* tgt = nullptr;   // [V0][3]
    std::vector<void*> all;
    ~NetBuffers() {
        for (void* p : all) cudaFree(p);
    }
};

Net::Net() = default;
Net::~Net() {
    for (auto* b : bufs_) delete b;
    cudaFree(p_); cudaFree(g_); cudaFree(m_); cudaFree(v_); cudaFree(wk_); cudaFree(wt_); cudaFree(loss_);
    cudaFree(tc_err_);
}

const std::vector<NetLayer>& Net::layers() {
    static const std::vector<NetLayer> L = make_layers();
    return L;
}

long long Net::param_count() {
    const auto& L = layers();
    return L.back().boff + L.back().cout + 1;   // + the identity gate g
}

pic_status Net::buffers(cudaStream_t, int n, int d, int h, int w, bool grads, NetBuffers** out, std::string* err) {
    for (auto* b : bufs_)
        if (b->dm0.N == n && b->dm0.D == d && b->dm0.H == h && b->dm0.W == w && (b->grads || !grads)) {
            *out = b;
            return PIC_OK;
        }
    auto* b = new NetBuffers();
    b->grads = grads;
    b->dm0 = {n, d, h, w};
    b->dm1 = {n, d / 2, h / 2, w / 2};
    b->dm2 = {n, d / 4, h / 4, w / 4};
    const long long V0 = b->dm0.vox(), V1 = b->dm1.vox(), V2 = b->dm2.vox();
    auto al = [&](void** p, size_t bytes) -> bool {
        if (cudaMalloc(p, bytes) != cudaSuccess) return false;
        b->all.push_back(*p);
        return true;
    };
    bool ok = true;
    auto a16 = [&](bf16** p, long long n_) { ok = ok && al((void**)p, sizeof(bf16) * (size_t)n_); };
    auto a32 = [&](float** p, long long n_) { ok = ok && al((void**)p, sizeof(float) * (size_t)n_); };
    a16(&b->x0, V0 * 16); a16(&b->e0a, V0 * 16); a16(&b->e0, V0 * 16); a16(&b->p1, V1 * 16);
    a16(&b->e1a, V1 * 32); a16(&b->e1, V1 * 32); a16(&b->p2, V2 * 32); a16(&b->e2a, V2 * 64); a16(&b->e2, V2 * 64);
    a16(&b->c1, V1 * 96); a16(&b->d1a, V1 * 32); a16(&b->d1, V1 * 32); a16(&b->c0, V0 * 48); a16(&b->d0a, V0 * 16);
    a16(&b->d0, V0 * 16); a32(&b->out, V0 * 16);
    if (grads) {
        a16(&b->g16, V0 * 48);
        a32(&b->A0, V0 * 48); a32(&b->B0, V0 * 48); a32(&b->S0, V0 * 16);
        a32(&b->A1, V1 * 96); a32(&b->B1, V1 * 96); a32(&b->S1, V1 * 32);
        a32(&b->A2, V2 * 64); a32(&b->B2, V2 * 64);
        a32(&b->tgt, V0 * 3);
    }
    if (!ok) {
        delete b;
        if (err) *err = "out of device memory for the network buffers";
        return PIC_ERR_NOMEM;
    }
    bufs_.push_back(b);
    *out = b;
    return PIC_OK;
}

void Net::refresh_bf16(cudaStream_t s) {
    for (const auto& l : layers())
        nn::k_weights_bf16<<<gs(27LL * l.cin * l.cout), 256, 0, s>>>(p_ + l.woff, (bf16*)wk_ + l.woff,
                                                                    (bf16*)wt_ + l.woff, l.cin, l.cout);
}

pic_status Net::init(cudaStream_t s, unsigned long long seed, std::string* err) {
    const long long n = param_count();
    if (!p_) {
        NCK(cudaMalloc(&p_, sizeof(float) * n));
        NCK(cudaMalloc(&g_, sizeof(float) * n));
        NCK(cudaMalloc(&m_, sizeof(float) * n));
        NCK(cudaMalloc(&v_, sizeof(float) * n));
        NCK(cudaMalloc(&wk_, sizeof(bf16) * n));
        NCK(cudaMalloc(&wt_, sizeof(bf16) * n));
        NCK(cudaMalloc(&loss_, sizeof(double)));
        NCK(cudaMalloc(&tc_err_, sizeof(int)));
        NCK(cudaMemsetAsync(tc_err_, 0, sizeof(int), s));
    }
    NCK(cudaMemsetAsync(p_, 0, sizeof(float) * n, s));
    NCK(cudaMemsetAsync(m_, 0, sizeof(float) * n, s));
    NCK(cudaMemsetAsync(v_, 0, sizeof(float) * n, s));
    NCK(cudaMemsetAsync(wt_, 0, sizeof(bf16) * n, s));
    for (size_t li = 0; li < layers().size(); ++li) {
        const auto& l = layers()[li];
        const int cin_real = li == E0A ? 6 : l.cin, cout_real = li == HEAD ? 3 : l.cout;
        // He-normal weights; the head starts at zero, so the untrained
        // preconditioner is the identity (z = r: plain GMRES)
        const float scale = li == HEAD ? 0.f : (float)std::sqrt(2.0 / (27.0 * cin_real));
        const long long nw = 27LL * l.cin * l.cout;
        k_he_init<<<gs(nw), 256, 0, s>>>(p_ + l.woff, nw, l.cin, l.cout, cin_real, cout_real, seed * 131 + li, scale);
    }
    adam_t_ = 0;
    gate_pending_ = true;   // g = 0 until training chooses its start
    refresh_bf16(s);
    NCK(cudaGetLastError());
    ready_ = true;
    return PIC_OK;
}

pic_status Net::set_params(cudaStream_t s, const float* host, std::string* err) {
    if (!p_) {
        pic_status st = init(s, 1, err);
        if (st != PIC_OK) return st;
    }
    const long long n = param_count();
    NCK(cudaMemcpyAsync(p_, host, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    gate_pending_ = false;   // the gate is part of the parameters
    NCK(cudaMemsetAsync(m_, 0, sizeof(float) * n, s));
    NCK(cudaMemsetAsync(v_, 0, sizeof(float) * n, s));
    adam_t_ = 0;
    refresh_bf16(s);
    NCK(cudaStreamSynchronize(s));
    ready_ = true;
    return PIC_OK;
}

pic_status Net::get_params(cudaStream_t s, float* host, std::string* err) {
    NCK(cudaMemcpyAsync(host, p_, sizeof(float) * param_count(), cudaMemcpyDeviceToHost, s));
    NCK(cudaStreamSynchronize(s));
    return PIC_OK;
}

pic_status Net::check_tc(cudaStream_t s, std::string* err) {
    int flag = 0;
    NCK(cudaMemcpyAsync(&flag, tc_err_, sizeof(int), cudaMemcpyDeviceToHost, s));
    NCK(cudaStreamSynchronize(s));
    if (flag) {
        cudaMemsetAsync(tc_err_, 0, sizeof(int), s);
        if (err) *err = "tensor-core convolution: an MMA completion wait ran out";
        return PIC_ERR_CUDA;
    }
    return PIC_OK;
}

void Net::forward(cudaStream_t s, NetBuffers& b) {
    const auto& L = layers();
    const bf16* wk = (const bf16*)wk_;
    auto cv = [&](int li, const bf16* x, bf16* y16, float* y32, Dims d) {
        const NetLayer& l = L[li];
        conv(s, l.cin, l.cout, x, wk + l.woff, p_ + l.boff, y16, y32, d, l.relu, tc_err_, wait_limit_);
    };
    cv(E0A, b.x0, b.e0a, nullptr, b.dm0);
    cv(E0B, b.e0a, b.e0, nullptr, b.dm0);
    nn::k_pool<<<gs(b.dm1.vox() * 2), 256, 0, s>>>(b.e0, b.p1, b.dm0, 16);
    cv(E1A, b.p1, b.e1a, nullptr, b.dm1);
    cv(E1B, b.e1a, b.e1, nullptr, b.dm1);
    nn::k_pool<<<gs(b.dm2.vox() * 4), 256, 0, s>>>(b.e1, b.p2, b.dm1, 32);
    cv(E2A, b.p2, b.e2a, nullptr, b.dm2);
    cv(E2B, b.e2a, b.e2, nullptr, b.dm2);
    nn::k_up_concat<<<gs(b.dm1.vox() * 12), 256, 0, s>>>(b.e2, b.e1, b.c1, b.dm1, 64, 32);
    cv(D1A, b.c1, b.d1a, nullptr, b.dm1);
    cv(D1B, b.d1a, b.d1, nullptr, b.dm1);
    nn::k_up_concat<<<gs(b.dm0.vox() * 6), 256, 0, s>>>(b.d1, b.e0, b.c0, b.dm0, 32, 16);
    cv(D0A, b.c0, b.d0a, nullptr, b.dm0);
    cv(D0B, b.d0a, b.d0, nullptr, b.dm0);
    cv(HEAD, b.d0, nullptr, b.out, b.dm0);
}

// Backward from the output gradient held in b.A0 ([V0][16] FP32); parameter
// gradients are added to g_.
void Net::backward(cudaStream_t s, NetBuffers& b) {
    const auto& L = layers();
    const bf16* wt = (const bf16*)wt_;
    // gpre = gy * relu'(y) in BF16, weight gradient, input gradient (FP32)
    auto back = [&](int li, const float* gy, const bf16* y, const bf16* x, float* gx, Dims d) {
        const NetLayer& l = L[li];
        const long long n = d.vox() * l.cout;
        nn::k_relu_bwd<<<gs(n), 256, 0, s>>>(gy, l.relu ? y : nullptr, b.g16, n);
        wgrad(s, l.cin, l.cout, x, b.g16, d, g_ + l.woff, g_ + l.boff);
        if (gx) conv(s, l.cout, l.cin, b.g16, wt + l.woff, nullptr, nullptr, gx, d, 0, tc_err_, wait_limit_);
    };
    back(HEAD, b.A0, nullptr, b.d0, b.B0, b.dm0);
    back(D0B, b.B0, b.d0, b.d0a, b.A0, b.dm0);
    back(D0A, b.A0, b.d0a, b.c0, b.B0, b.dm0);
    nn::k_up_concat_bwd<<<gs(b.dm0.vox() * 16), 256, 0, s>>>(b.B0, b.A1, b.S0, b.dm0, 32, 16);
    back(D1B, b.A1, b.d1, b.d1a, b.B1, b.dm1);
    back(D1A, b.B1, b.d1a, b.c1, b.A1, b.dm1);
    nn::k_up_concat_bwd<<<gs(b.dm1.vox() * 32), 256, 0, s>>>(b.A1, b.A2, b.S1, b.dm1, 64, 32);
    back(E2B, b.A2, b.e2, b.e2a, b.B2, b.dm2);
    back(E2A, b.B2, b.e2a, b.p2, b.A2, b.dm2);
    nn::k_pool_bwd_add<<<gs(b.dm1.vox() * 32), 256, 0, s>>>(b.A2, b.S1, b.dm1, 32);
    back(E1B, b.S1, b.e1, b.e1a, b.B1, b.dm1);
    back(E1A, b.B1, b.e1a, b.p1, b.A1, b.dm1);
    nn::k_pool_bwd_add<<<gs(b.dm0.vox() * 16), 256, 0, s>>>(b.A1, b.S0, b.dm0, 16);
    back(E0B, b.S0, b.e0, b.e0a, b.A0, b.dm0);
    back(E0A, b.A0, b.e0a, b.x0, nullptr, b.dm0);
}

static bool dims_ok(int n, int d, int h, int w) { return n >= 1 && d >= 4 && h >= 4 && w >= 4 && d % 4 == 0 && h % 4 == 0 && w % 4 == 0; }

pic_status Net::forward_host(cudaStream_t s, int n, int d, int h, int w, const float* x0, float* out,
                             std::string* err) {
    if (!ready_) { if (err) *err = "network not initialised"; return PIC_ERR_STATE; }
    if (!dims_ok(n, d, h, w)) { if (err) *err = "network dims must be multiples of 4"; return PIC_ERR_ARG; }
    NetBuffers* b = nullptr;
    pic_status st = buffers(s, n, d, h, w, false, &b, err);
    if (st != PIC_OK) return st;
    const long long V = b->dm0.vox();
    float* tmp = nullptr;
    NCK(cudaMalloc(&tmp, sizeof(float) * V * 16));
    cudaMemcpyAsync(tmp, x0, sizeof(float) * V * 16, cudaMemcpyHostToDevice, s);
    k_f32_to_bf16<<<gs(V * 16), 256, 0, s>>>(tmp, b->x0, V * 16);
    forward(s, *b);
    cudaMemcpyAsync(out, b->out, sizeof(float) * V * 16, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    cudaFree(tmp);
    NCK(e);
    NCK(cudaGetLastError());
    return check_tc(s, err);
}

pic_status Net::loss_grad_host(cudaStream_t s, int n, int d, int h, int w, const float* x0, const float* target,
                               double* loss, float* grad, std::string* err) {
    if (!ready_) { if (err) *err = "network not initialised"; return PIC_ERR_STATE; }
    if (!dims_ok(n, d, h, w)) { if (err) *err = "network dims must be multiples of 4"; return PIC_ERR_ARG; }
    NetBuffers* b = nullptr;
    pic_status st = buffers(s, n, d, h, w, true, &b, err);
    if (st != PIC_OK) return st;
    const long long V = b->dm0.vox();
    NCK(cudaMemcpyAsync(b->A0, x0, sizeof(float) * V * 16, cudaMemcpyHostToDevice, s));
    k_f32_to_bf16<<<gs(V * 16), 256, 0, s>>>(b->A0, b->x0, V * 16);
    NCK(cudaMemcpyAsync(b->tgt, target, sizeof(float) * V * 3, cudaMemcpyHostToDevice, s));
    forward(s, *b);
    NCK(cudaMemsetAsync(loss_, 0, sizeof(double), s));
    NCK(cudaMemsetAsync(g_, 0, sizeof(float) * param_count(), s));
    nn::k_mse<<<gs(V * 16), 256, 0, s>>>(b->out, b->tgt, b->A0, V, 16, 3, 1.f, loss_);
    backward(s, *b);
    NCK(cudaMemcpyAsync(loss, loss_, sizeof(double), cudaMemcpyDeviceToHost, s));
    NCK(cudaMemcpyAsync(grad, g_, sizeof(float) * param_count(), cudaMemcpyDeviceToHost, s));
    NCK(cudaStreamSynchronize(s));
    NCK(cudaGetLastError());
    return check_tc(s, err);
}

pic_status Net::apply(cudaStream_t s, const GridP& g, const double* mu, const double* v, double* z, double* scal,
                      double* partials, std::string* err) {
    NetBuffers* b = nullptr;
    pic_status st = buffers(s, 1, g.nz, g.ny, g.nx, false, &b, err);
    if (st != PIC_OK) return st;
    const long long L = 3 * g.N;
    launch_dot(s, v, v, L, partials, red_blocks(L), scal, 1);
    double nv = 0;
    NCK(cudaMemcpyAsync(&nv, scal, sizeof(double), cudaMemcpyDeviceToHost, s));
    st = check_tc(s, err);   // also waits for the norm
    if (st != PIC_OK) return st;
    if (!(nv > 0) || !std::isfinite(nv)) {
        NCK(cudaMemsetAsync(z, 0, sizeof(double) * L, s));
        return PIC_OK;
    }
    const double sc = nv / std::sqrt((double)L);
    k_pack_box<<<gs(g.N), 256, 0, s>>>(v, 1.0 / sc, mu, b->x0, g.N);
    forward(s, *b);
    k_unpack_box<<<gs(g.N), 256, 0, s>>>(b->out, sc, v, p_ + param_count() - 1, z, g.N);
    NCK(cudaGetLastError());
    return PIC_OK;
}

pic_status Net::train(cudaStream_t s, const GridP& g, const double* mu, const pic_train_opts& o, pic_train_info* info,
                      double* partials, std::string* err) {
    if (!ready_) { if (err) *err = "network not initialised"; return PIC_ERR_STATE; }
    const int nb = o.batch > 0 ? o.batch : 1;
    if (g.nx % 4 || g.ny % 4 || g.nz % 4) {
        if (err) *err = "box axes must be multiples of 4";
        return PIC_ERR_ARG;
    }
    NetBuffers* b = nullptr;
    pic_status st = buffers(s, nb, g.nz, g.ny, g.nx, true, &b, err);
    if (st != PIC_OK) return st;
    const long long L = 3 * g.N;
    double *r = nullptr, *r2 = nullptr, *z = nullptr, *e = nullptr, *wm = nullptr, *scal = nullptr;
    std::vector<void*> tmp;
    auto al = [&](double** p, size_t n) -> bool {
        if (cudaMalloc((void**)p, sizeof(double) * n) != cudaSuccess) return false;
        tmp.push_back(*p);
        return true;
    };
    auto cleanup = [&]() { for (void* p : tmp) cudaFree(p); };
    float *best_p = nullptr, *prev_p = nullptr;
    auto alf = [&](float** p, size_t n) -> bool {
        if (cudaMalloc((void**)p, sizeof(float) * n) != cudaSuccess) return false;
        tmp.push_back(*p);
        return true;
    };
    if (!al(&r, (size_t)L * nb) || !al(&r2, L) || !al(&z, L) || !al(&e, L) || !al(&wm, L) ||
        !al(&scal, 4 + (size_t)nb) || !alf(&best_p, param_count()) || !alf(&prev_p, param_count())) {
        cleanup();
        if (err) *err = "out of device memory for training";
        return PIC_ERR_NOMEM;
    }
    const OpCoef oc = make_opcoef(g);
    const long long V = g.N;   // voxels per field
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    unsigned long long rng = o.seed * 0x9E3779B97F4A7C15ull + 12345;
    auto next = [&]() {
        rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17;   // xorshift64
        return rng;
    };
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    double first = 0, last = 0, best = INFINITY;
    // every kCheck steps (and at both ends) the batch loss is read; the
    // parameters of the lowest checked loss are kept on the device and
    // restored at the end if the run degraded from there (Adam at a constant
    // rate can diverge late in long runs)
    constexpr int kCheck = 50;
    const int steps = o.steps > 0 ? o.steps : 1;
    for (int it = 0; it < steps; ++it) {
        // nb random fields r (white noise after 0 .. smooth_max binomial
        // passes), each scaled to unit rms and packed with the mu diagonal
        for (int q = 0; q < nb; ++q) {
            double* rq = r + (size_t)q * L;
            k_noise<<<gs(L), 256, 0, s>>>(rq, L, (o.seed * 1000003ull + it) * 64 + q);
            const int passes = o.smooth_max > 0 ? (int)(next() % (unsigned long long)(o.smooth_max + 1)) : 0;
            for (int k = 0; k < passes; ++k) {
                k_smooth<<<gs(L), 256, 0, s>>>(g, rq, r2);
                cudaMemcpyAsync(rq, r2, sizeof(double) * L, cudaMemcpyDeviceToDevice, s);
            }
            launch_dot(s, rq, rq, L, partials, red_blocks(L), scal, 1);
            k_rescale_by_norm<<<gs(L), 256, 0, s>>>(rq, L, scal);
            k_pack_box<<<gs(V), 256, 0, s>>>(rq, 1.0, mu, b->x0 + (size_t)q * V * 16, V);
        }
        if (gate_pending_) {
            // a fresh network starts from the identity (g = 1) where the
            // identity preconditioner already reduces the residual of the
            // first batch's field, |A r - r| < |r|, else from zero (g = 0)
            cudaMemsetAsync(loss_, 0, sizeof(double), s);
            launch_maxwell_apply(s, g, oc, mu, r, e, wm);
            k_sub_loss<<<gs(L), 256, 0, s>>>(e, r, L, 1.0 / (double)L, loss_);
            double l1 = 0;
            cudaMemcpyAsync(&l1, loss_, sizeof(double), cudaMemcpyDeviceToHost, s);
            cudaError_t ce = cudaStreamSynchronize(s);
            if (ce != cudaSuccess) { cleanup(); NCK(ce); }
            const float g0 = l1 < 1.0 ? 1.0f : 0.0f;
            cudaMemcpyAsync(p_ + param_count() - 1, &g0, sizeof(float), cudaMemcpyHostToDevice, s);
            cudaStreamSynchronize(s);
            gate_pending_ = false;
        }
        forward(s, *b);
        // residual loss L = mean_q |A z_q - r_q|^2 / |r_q|^2 (|r_q|^2 = 3N),
        // z_q = g r_q + net(r_q); dL/dnet_q = 2 A^T (A z_q - r_q) / (3N nb),
        // dL/dg = sum_q <dL/dz_q, r_q>
        const float* gate = p_ + param_count() - 1;
        cudaMemsetAsync(loss_, 0, sizeof(double), s);
        for (int q = 0; q < nb; ++q) {
            const double* rq = r + (size_t)q * L;
            k_unpack_box<<<gs(V), 256, 0, s>>>(b->out + (size_t)q * V * 16, 1.0, rq, gate, z, V);
            launch_maxwell_apply(s, g, oc, mu, z, e, wm);
            k_sub_loss<<<gs(L), 256, 0, s>>>(e, rq, L, 1.0 / ((double)L * nb), loss_);
            launch_maxwell_apply_t(s, g, oc, mu, e, z);
            k_pack_grad<<<gs(V), 256, 0, s>>>(z, 2.0 / ((double)L * nb), b->A0 + (size_t)q * V * 16, V);
            launch_dot(s, z, rq, L, partials, red_blocks(L), scal + 4 + q, 0);
        }
        cudaMemsetAsync(g_, 0, sizeof(float) * param_count(), s);
        backward(s, *b);
        k_gate_grad<<<1, 1, 0, s>>>(scal + 4, nb, 2.0 / ((double)L * nb), g_ + param_count() - 1);
        const bool check = it == 0 || it == steps - 1 || it % kCheck == kCheck - 1;
        if (check) cudaMemcpyAsync(prev_p, p_, sizeof(float) * param_count(), cudaMemcpyDeviceToDevice, s);
        ++adam_t_;
        const float c1 = (float)(o.lr / (1.0 - std::pow((double)b1, adam_t_)));
        const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, adam_t_)));
        nn::k_adam<<<gs(param_count()), 256, 0, s>>>(p_, g_, m_, v_, param_count(), b1, b2, eps, c1, c2);
        refresh_bf16(s);
        if (check) {
            double lv = 0;
            cudaMemcpyAsync(&lv, loss_, sizeof(double), cudaMemcpyDeviceToHost, s);
            cudaError_t ce = cudaStreamSynchronize(s);
            if (ce != cudaSuccess) { cleanup(); NCK(ce); }
            if (it == 0) first = lv;
            last = lv;
            if (std::isfinite(lv) && lv < best) {
                best = lv;
                // the loss was measured before this step's update: keep the
                // parameters that produced it
                cudaMemcpyAsync(best_p, prev_p, sizeof(float) * param_count(), cudaMemcpyDeviceToDevice, s);
            }
        }
    }
    if (!(last <= best) && std::isfinite(best)) {
        cudaMemcpyAsync(p_, best_p, sizeof(float) * param_count(), cudaMemcpyDeviceToDevice, s);
        refresh_bf16(s);
        last = best;
    }
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaError_t ce = cudaGetLastError();
    cleanup();
    NCK(ce);
    if (info) {
        info->first_loss = first;
        info->last_loss = last;
        info->seconds = ms * 1e-3;
        info->steps = steps;
    }
    if (!std::isfinite(last)) {
        if (err) *err = "training diverged";
        return PIC_ERR_NUMERIC;
    }
    return check_tc(s, err);
}

// ---- recorded triples ---------------------------------------------------
TripleStore::~TripleStore() { release(); }

void TripleStore::release() {
    cudaFree(data);
    data = nullptr;
    cap = count = 0;
    N = 0;
    xx.clear();
}

pic_status TripleStore::reserve(int capacity, long long n, std::string* err) {
    release();
    if (capacity <= 0) return PIC_OK;
    NCK(cudaMalloc(&data, sizeof(float) * 15 * (size_t)n * (size_t)capacity));
    cap = capacity;
    N = n;
    return PIC_OK;
}

pic_status TripleStore::add(cudaStream_t s, const double* b, const double* mu, const double* x, double* scal,
                            double* partials, std::string* err) {
    if (!data || count >= cap) return PIC_OK;
    float* dst = data + (size_t)count * 15 * (size_t)N;
    const long long L = 3 * N;
    k_d2f<<<gs(L), 256, 0, s>>>(b, dst, L);
    k_d2f<<<gs(3 * L), 256, 0, s>>>(mu, dst + L, 3 * L);
    k_d2f<<<gs(L), 256, 0, s>>>(x, dst + 4 * L, L);
    launch_dot(s, b, b, L, partials, red_blocks(L), scal, 0);
    launch_dot(s, x, x, L, partials, red_blocks(L), scal + 1, 0);
    double h[2] = {0, 0};
    NCK(cudaMemcpyAsync(h, scal, sizeof(h), cudaMemcpyDeviceToHost, s));
    NCK(cudaStreamSynchronize(s));
    xx.push_back(h[0] > 0 ? h[1] / h[0] : 0.0);
    ++count;
    return PIC_OK;
}

pic_status Net::train_triples(cudaStream_t s, const GridP& g, const TripleStore& ts, const pic_train_opts& o,
                              pic_train_info* info, double* partials, std::string* err) {
    if (!ready_) { if (err) *err = "network not initialised"; return PIC_ERR_STATE; }
    if (ts.count < 1 || ts.N != g.N) { if (err) *err = "no recorded triples of this box"; return PIC_ERR_STATE; }
    const int nb = o.batch > 0 ? o.batch : 1;
    if (g.nx % 4 || g.ny % 4 || g.nz % 4) {
        if (err) *err = "box axes must be multiples of 4";
        return PIC_ERR_ARG;
    }
    NetBuffers* b = nullptr;
    pic_status st = buffers(s, nb, g.nz, g.ny, g.nx, true, &b, err);
    if (st != PIC_OK) return st;
    const long long L = 3 * g.N, V = g.N;
    std::vector<void*> tmp;
    auto cleanup = [&]() { for (void* p : tmp) cudaFree(p); };
    auto al = [&](void** p, size_t bytes) -> bool {
        if (cudaMalloc(p, bytes) != cudaSuccess) return false;
        tmp.push_back(*p);
        return true;
    };
    double *bb = nullptr, *xb = nullptr, *mb = nullptr, *z = nullptr, *e = nullptr, *es = nullptr, *t = nullptr,
           *wm = nullptr, *scal = nullptr;
    float *best_p = nullptr, *prev_p = nullptr;
    const size_t d8 = sizeof(double);
    if (!al((void**)&bb, d8 * L * nb) || !al((void**)&xb, d8 * L * nb) || !al((void**)&mb, d8 * 3 * L * nb) ||
        !al((void**)&z, d8 * L) || !al((void**)&e, d8 * L) || !al((void**)&es, d8 * L) || !al((void**)&t, d8 * L) ||
        !al((void**)&wm, d8 * L) || !al((void**)&scal, d8 * (4 + (size_t)nb)) ||
        !al((void**)&best_p, sizeof(float) * param_count()) || !al((void**)&prev_p, sizeof(float) * param_count())) {
        cleanup();
        if (err) *err = "out of device memory for training";
        return PIC_ERR_NOMEM;
    }
    const OpCoef oc = make_opcoef(g);
    const double ws = std::min(std::max(o.supervised_weight, 0.0), 1.0), wr = 1.0 - ws;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    unsigned long long rng = o.seed * 0x9E3779B97F4A7C15ull + 777;
    auto next = [&]() {
        rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17;   // xorshift64
        return rng;
    };
    if (gate_pending_) {   // the recorded solutions decide nothing here: start from the identity
        const float g1 = 1.0f;
        cudaMemcpyAsync(p_ + param_count() - 1, &g1, sizeof(float), cudaMemcpyHostToDevice, s);
        gate_pending_ = false;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    double first = 0, last = 0, best = INFINITY;
    constexpr int kCheck = 50;
    const int steps = o.steps > 0 ? o.steps : 1;
    std::vector<int> pick(nb);
    const float* gate = p_ + param_count() - 1;
    for (int it = 0; it < steps; ++it) {
        for (int q = 0; q < nb; ++q) {
            pick[q] = (int)(next() % (unsigned long long)ts.count);
            const float* src = ts.data + (size_t)pick[q] * 15 * (size_t)ts.N;
            double* bq = bb + (size_t)q * L;
            double* xq = xb + (size_t)q * L;
            double* mq = mb + (size_t)q * 3 * L;
            k_f2d<<<gs(L), 256, 0, s>>>(src, bq, L);
            k_f2d<<<gs(3 * L), 256, 0, s>>>(src + L, mq, 3 * L);
            k_f2d<<<gs(L), 256, 0, s>>>(src + 4 * L, xq, L);
            // b to unit rms, x by the same factor (A x = b is linear)
            launch_dot(s, bq, bq, L, partials, red_blocks(L), scal, 1);
            k_rescale_by_norm<<<gs(L), 256, 0, s>>>(bq, L, scal);
            k_rescale_by_norm<<<gs(L), 256, 0, s>>>(xq, L, scal);
            k_pack_box<<<gs(V), 256, 0, s>>>(bq, 1.0, mq, b->x0 + (size_t)q * V * 16, V);
        }
        forward(s, *b);
        cudaMemsetAsync(loss_, 0, sizeof(double), s);
        for (int q = 0; q < nb; ++q) {
            const double* bq = bb + (size_t)q * L;
            const double* xq = xb + (size_t)q * L;
            const double* mq = mb + (size_t)q * 3 * L;
            const double xx = ts.xx[pick[q]] > 0 ? ts.xx[pick[q]] : 1.0;   // |x|^2 / |b|^2, |b|^2 = L now
            k_unpack_box<<<gs(V), 256, 0, s>>>(b->out + (size_t)q * V * 16, 1.0, bq, gate, z, V);
            // residual part: e = A z - b, t = A^T e
            launch_maxwell_apply(s, g, oc, mq, z, e, wm);
            k_sub_loss<<<gs(L), 256, 0, s>>>(e, bq, L, wr / ((double)L * nb), loss_);
            launch_maxwell_apply_t(s, g, oc, mq, e, t);
            // supervised part: es = z - x
            cudaMemcpyAsync(es, z, sizeof(double) * L, cudaMemcpyDeviceToDevice, s);
            k_sub_loss<<<gs(L), 256, 0, s>>>(es, xq, L, ws / (xx * (double)L * nb), loss_);
            // dL/dz = 2 (1 - w) A^T e / (L nb) + 2 w (z - x) / (|x|^2 nb)
            k_axpby<<<gs(L), 256, 0, s>>>(t, es, 2.0 * wr / ((double)L * nb), 2.0 * ws / (xx * (double)L * nb), L);
            k_pack_grad<<<gs(V), 256, 0, s>>>(t, 1.0, b->A0 + (size_t)q * V * 16, V);
            launch_dot(s, t, bq, L, partials, red_blocks(L), scal + 4 + q, 0);
        }
        cudaMemsetAsync(g_, 0, sizeof(float) * param_count(), s);
        backward(s, *b);
        k_gate_grad<<<1, 1, 0, s>>>(scal + 4, nb, 1.0, g_ + param_count() - 1);
        const bool check = it == 0 || it == steps - 1 || it % kCheck == kCheck - 1;
        if (check) cudaMemcpyAsync(prev_p, p_, sizeof(float) * param_count(), cudaMemcpyDeviceToDevice, s);
        ++adam_t_;
        const float c1 = (float)(o.lr / (1.0 - std::pow((double)b1, adam_t_)));
        const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, adam_t_)));
        nn::k_adam<<<gs(param_count()), 256, 0, s>>>(p_, g_, m_, v_, param_count(), b1, b2, eps, c1, c2);
        refresh_bf16(s);
        if (check) {
            double lv = 0;
            cudaMemcpyAsync(&lv, loss_, sizeof(double), cudaMemcpyDeviceToHost, s);
            cudaError_t ce = cudaStreamSynchronize(s);
            if (ce != cudaSuccess) { cleanup(); NCK(ce); }
            if (it == 0) first = lv;
            last = lv;
            if (std::isfinite(lv) && lv < best) {
                best = lv;
                cudaMemcpyAsync(best_p, prev_p, sizeof(float) * param_count(), cudaMemcpyDeviceToDevice, s);
            }
        }
    }
    if (!(last <= best) && std::isfinite(best)) {
        cudaMemcpyAsync(p_, best_p, sizeof(float) * param_count(), cudaMemcpyDeviceToDevice, s);
        refresh_bf16(s);
        last = best;
    }
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaError_t ce = cudaGetLastError();
    cleanup();
    NCK(ce);
    if (info) {
        info->first_loss = first;
        info->last_loss = last;
        info->seconds = ms * 1e-3;
        info->steps = steps;
    }
    if (!std::isfinite(last)) {
        if (err) *err = "training diverged";
        return PIC_ERR_NUMERIC;
    }
    return check_tc(s, err);
}

}  // namespace pic
