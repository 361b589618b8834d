// nn.hpp -- the learned right preconditioner z = g r + s net(r / s, mu
// diagonal), g a trained gate (the last parameter; training starts it at 1
// where the identity already reduces the residual, else at 0): a 3-level
// 3x3x3-convolution encoder-decoder (16/32/64
// channels, 6 input channels: residual and mu diagonal; 3 output channels:
// the correction), linear (no activation: with mu fixed during a solve the
// preconditioner is a fixed linear operator, as flexible GMRES converges
// best with), BF16 activations with FP32 accumulation, trained on the
// device with its own forward, backward and Adam kernels.  The FP64 numpy
// restatement in the oracle defines the same network and parameter layout.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "../../include/picpp_gb300.h"
#include "common.cuh"

namespace pic {

struct NetLayer {
    const char* name;
    int cin, cout, relu;   // relu: 0 for every layer of this network
    long long woff, boff;   // offsets of W[27][cout][cin] and b[cout] in the parameter vector
};

struct NetBuffers;   // activations and gradients of one shape (nn.cu)

// (right-hand side b, mu, solution x) triples of plain field solves, kept in
// FP32 on the device for training the network: the first `cap` recorded.
struct TripleStore {
    int cap = 0, count = 0;
    long long N = 0;             // cells of the box they come from
    float* data = nullptr;       // per triple: b [3N], mu [9N], x [3N]
    std::vector<double> xx;      // |x|^2 / |b|^2 of each triple
    ~TripleStore();
    void release();
    pic_status reserve(int capacity, long long n, std::string* err);
    // stores one more triple unless full; scal, partials: reduction scratch
    pic_status add(cudaStream_t s, const double* b, const double* mu, const double* x, double* scal,
                   double* partials, std::string* err);
};



class Net {
public:
    Net();
    ~Net();
    static long long param_count();
    static const std::vector<NetLayer>& layers();

    pic_status init(cudaStream_t s, unsigned long long seed, std::string* err);
    pic_status set_params(cudaStream_t s, const float* host, std::string* err);
    pic_status get_params(cudaStream_t s, float* host, std::string* err);
    bool ready() const { return ready_; }
    // polls of the convolutions' MMA-completion wait before it gives up and
    // reports an error (0: the built-in bound)
    void set_wait_limit(unsigned polls) { wait_limit_ = polls; }
    // waits for the stream; an error if a convolution reported a timed-out wait
    pic_status check_tc(cudaStream_t s, std::string* err);

    // x0: [n][d][h][w][16] BF16 on the device is packed by the callers below.
    // Forward on host FP32 input (channels 16), output [..][16] FP32 to host.
    pic_status forward_host(cudaStream_t s, int n, int d, int h, int w, const float* x0, float* out, std::string* err);
    // Loss and parameter gradient for host input and target [..][3].
    pic_status loss_grad_host(cudaStream_t s, int n, int d, int h, int w, const float* x0, const float* target,
                              double* loss, float* grad, std::string* err);
    // z = g v + s * net(v / s, mu diagonal) on the box (FP64 planar vectors of 3N).
    pic_status apply(cudaStream_t s, const GridP& g, const double* mu, const double* v, double* z, double* scal,
                     double* partials, std::string* err);
    // Training on the box's operator A(mu): random fields r of unit rms
    // (white noise after 0 .. smooth_max binomial passes), loss
    // |A z - r|^2 / |r|^2 with z = g r + net(r, mu diagonal); its gradient
    // 2 A^T (A z - r) / |r|^2 (k_maxwell_apply_t) seeds the backward pass
    // and, dotted with r, gives the gate's.
    pic_status train(cudaStream_t s, const GridP& g, const double* mu, const pic_train_opts& o, pic_train_info* info,
                     double* partials, std::string* err);
    // Training on recorded triples (b, mu, x) of the box g: batches of
    // o.batch triples, loss w |z - x|^2 / |x|^2 + (1 - w) |A(mu) z - b|^2 / |b|^2
    // with z = g b + net(b, mu diagonal) and w = o.supervised_weight, every
    // triple scaled to a unit-rms right-hand side.
    pic_status train_triples(cudaStream_t s, const GridP& g, const TripleStore& ts, const pic_train_opts& o,
                             pic_train_info* info, double* partials, std::string* err);

private:
    pic_status buffers(cudaStream_t s, int n, int d, int h, int w, bool grads, NetBuffers** out, std::string* err);
    void refresh_bf16(cudaStream_t s);
    void forward(cudaStream_t s, NetBuffers& b);
    void backward(cudaStream_t s, NetBuffers& b);   // from b.out gradient in b's loss-gradient buffer
    float *p_ = nullptr, *g_ = nullptr, *m_ = nullptr, *v_ = nullptr;
    void* wk_ = nullptr;   // BF16 forward weights, per layer at woff
    void* wt_ = nullptr;   // BF16 flipped/transposed weights
    double* loss_ = nullptr;
    int* tc_err_ = nullptr;   // set by a convolution whose MMA completion wait ran out
    int adam_t_ = 0;
    unsigned wait_limit_ = 0;
    bool gate_pending_ = false;   // fresh network: training picks the gate's start
    bool ready_ = false;
    std::vector<NetBuffers*> bufs_;
};

}  // namespace pic
