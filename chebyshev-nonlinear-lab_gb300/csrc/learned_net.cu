// learned_net.cu — the learned preconditioner's network: a 4-level 3D convolutional U-Net on the
// multigrid hierarchy (levels n0, (n0-1)/2, ...), BF16 activations in the 8-channel plane layout,
// convolutions and their input gradients on the tensor cores (learned_conv.cuh), weight gradients
// in FP32 on the CUDA cores, FP32 master weights updated by Adam.
//
//   level 0 (n0):  e0a 16->16, e0b 16->16 = s0                 (input: 3 feature channels of 16)
//   level 1:       e1a 16->32, e1b 32->32 = s1                  (R s0 in)
//   level 2:       e2a 32->32, e2b 32->32 = s2                  (R s1 in)
//   level 3:       e3a 32->32, e3b 32->32                       (R s2 in)
//   up:            d2 32->32 on P e3b + s2; d1 32->16 on P d2 + s1; d0a 16->16, d0b 16->16 on P d1 + s0
// Every convolution is 3x3x3 with bias and ReLU except d0b, whose channel 0 is the output.  R and P
// are the multigrid's full-weighting restriction and trilinear prolongation applied per channel;
// their adjoints are P / 8 and 8 R.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "learned_conv.cuh"
#include "numa_internal.hpp"

namespace numa::gpu {

// kernels and launches of learned.cu
void conv3d_tc(Context& ctx, const VoxGrid& g, int cin, int cout, const uint4* in, const uint4* wg, const float* bias,
               uint4* out, float* out32, int relu, unsigned* err);
void pack_weights(Context& ctx, const float* w, __nv_bfloat16* wg, int cin, int cout, bool flip);
void planes_restrict(Context& ctx, const uint4* fine, uint4* coarse, const VoxGrid& gf, const VoxGrid& gc, int C,
                     float scale);
void planes_prolong(Context& ctx, const uint4* coarse, const uint4* add, uint4* out, const VoxGrid& gc,
                    const VoxGrid& gf, int C, float scale, bool accumulate);
void planes_relu_mask(Context& ctx, uint4* g, const uint4* y, const VoxGrid& gr, int C);
void conv_dw(Context& ctx, const VoxGrid& gr, int cin, int cout, const uint4* x, const uint4* g, float* dw, float* db,
             DeviceArray<float>& part, unsigned* err);
void planes_features(Context& ctx, const float* r, const float* c, const float* z, const float* scales, uint4* planes,
                     const VoxGrid& gr);
void planes_loss_grad(Context& ctx, const float* y32, const float* t, uint4* g, const VoxGrid& gr, float* loss);
void adam_step(Context& ctx, float* w, const float* g, float* m, float* v, size_t n, float lr, int t);

namespace {

struct LayerSpec {
    int cin, cout, level;
    bool relu;
};
// e0a e0b e1a e1b e2a e2b e3a e3b d2 d1 d0a d0b
constexpr LayerSpec kLayers[] = {{16, 16, 0, true},  {16, 16, 0, true},  {16, 32, 1, true},  {32, 32, 1, true},
                                 {32, 32, 2, true},  {32, 32, 2, true},  {32, 32, 3, true},  {32, 32, 3, true},
                                 {32, 32, 2, true},  {32, 16, 1, true},  {16, 16, 0, true},  {16, 16, 0, false}};
constexpr int kNumLayers = 12;
enum { E0A, E0B, E1A, E1B, E2A, E2B, E3A, E3B, D2, D1, D0A, D0B };

}  // namespace

// A tensor in the plane layout on one level.
struct PlaneTensor {
    DeviceArray<uint4> buf;
    int C = 0, level = 0;
    void init(const VoxGrid& g, int channels, int lvl, cudaStream_t s) {
        C = channels;
        level = lvl;
        buf.resize((size_t)(channels / 8) * g.rows);
        NUMA_CUDA(cudaMemsetAsync(buf.p, 0, buf.n * sizeof(uint4), s));
    }
    uint4* p() { return buf.p; }
};

class LearnedNet {
public:
    LearnedNet(Context& ctx, int n0, uint64_t seed);
    int n0() const { return n0_; }
    size_t num_params() const { return nparams_; }
    const VoxGrid& grid(int l) const { return g_[l]; }
    // Host copies of the FP32 master parameters (layer order: W [27][cin][cout], then b [cout]).
    void get_params(float* host) const;
    void set_params(const float* host);
    // out32 [n0^3][16] (channel 0 = the correction) from the 16-channel feature planes.
    void forward(const uint4* in, float* out32);
    // One training step's gradient: forward, loss against t (n0^3), backward; gradients are summed
    // into grad_ (zeroed by zero_grad).  Returns nothing: the loss accumulates in *loss_dev.
    void loss_and_backward(const uint4* in, const float* t, float* loss_dev);
    void zero_grad();
    void adam(float lr);
    float* grad() { return grad_.p; }
    uint4* feature_planes() { return feat_.p(); }
    float* out32() { return out32_.p; }
    void check_errors();

private:
    void repack();
    void conv(int l, const uint4* in, uint4* out, float* o32);
    void conv_adj(int l, const uint4* g, uint4* out);
    void dw(int l, const uint4* x, const uint4* g);
    Context& ctx_;
    int n0_;
    VoxGrid g_[4];
    size_t nparams_ = 0, woff_[kNumLayers], boff_[kNumLayers];
    DeviceArray<float> params_, grad_, m_, v_;
    DeviceArray<__nv_bfloat16> wf_[kNumLayers], wb_[kNumLayers];
    DeviceArray<unsigned> err_;
    DeviceArray<float> dw_part_;  // per-CTA partials of the tensor-core weight gradient
    DeviceArray<float> out32_, gout32_;
    int step_ = 0;
    // activations
    PlaneTensor feat_, a_e0a_, s0_, r1_, a_e1a_, s1_, r2_, a_e2a_, s2_, r3_, a_e3a_, a_e3b_, u2_, a_d2_, u1_, a_d1_,
        u0_, a_d0a_;
    // gradients
    PlaneTensor g_out_, g_t0_, g_u0_, g_d1_, g_u1_, g_d2_, g_u2_, g_e3b_, g_e3a_, g_r3_, g_e2a_, g_r2_, g_e1a_, g_r1_,
        g_e0a_;
    bool packed_ = false;
};

LearnedNet::LearnedNet(Context& ctx, int n0, uint64_t seed) : ctx_(ctx), n0_(n0) {
    if (!(n0 == 15 || n0 == 31 || n0 == 63))
        throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "learned network: base grid must be 15, 31 or 63");
    int n = n0;
    for (int l = 0; l < 4; ++l) {
        g_[l] = make_voxgrid(n);
        n = (n - 1) / 2;
    }
    for (int l = 0; l < kNumLayers; ++l) {
        woff_[l] = nparams_;
        nparams_ += (size_t)27 * kLayers[l].cin * kLayers[l].cout;
        boff_[l] = nparams_;
        nparams_ += kLayers[l].cout;
        wf_[l].resize((size_t)27 * kLayers[l].cin * kLayers[l].cout);
        wb_[l].resize((size_t)27 * kLayers[l].cin * kLayers[l].cout);
    }
    // He-normal initialisation (std sqrt(2 / fan_in)), biases zero; the output layer scaled by 0.1
    std::vector<float> h(nparams_, 0.0f);
    std::mt19937_64 rng(seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    for (int l = 0; l < kNumLayers; ++l) {
        const double sd = std::sqrt(2.0 / (27.0 * kLayers[l].cin)) * (l == D0B ? 0.1 : 1.0);
        const size_t cnt = (size_t)27 * kLayers[l].cin * kLayers[l].cout;
        for (size_t i = 0; i < cnt; ++i) h[woff_[l] + i] = (float)(sd * nd(rng));
    }
    params_.resize(nparams_);
    grad_.resize(nparams_);
    m_.resize(nparams_);
    v_.resize(nparams_);
    NUMA_CUDA(cudaMemcpyAsync(params_.p, h.data(), nparams_ * sizeof(float), cudaMemcpyHostToDevice, ctx_.stream));
    NUMA_CUDA(cudaMemsetAsync(m_.p, 0, nparams_ * sizeof(float), ctx_.stream));
    NUMA_CUDA(cudaMemsetAsync(v_.p, 0, nparams_ * sizeof(float), ctx_.stream));
    err_.resize(1);
    NUMA_CUDA(cudaMemsetAsync(err_.p, 0, sizeof(unsigned), ctx_.stream));
    const size_t N0 = (size_t)n0 * n0 * n0;
    out32_.resize(N0 * 16);
    cudaStream_t s = ctx_.stream;
    feat_.init(g_[0], 16, 0, s);
    a_e0a_.init(g_[0], 16, 0, s);
    s0_.init(g_[0], 16, 0, s);
    r1_.init(g_[1], 16, 1, s);
    a_e1a_.init(g_[1], 32, 1, s);
    s1_.init(g_[1], 32, 1, s);
    r2_.init(g_[2], 32, 2, s);
    a_e2a_.init(g_[2], 32, 2, s);
    s2_.init(g_[2], 32, 2, s);
    r3_.init(g_[3], 32, 3, s);
    a_e3a_.init(g_[3], 32, 3, s);
    a_e3b_.init(g_[3], 32, 3, s);
    u2_.init(g_[2], 32, 2, s);
    a_d2_.init(g_[2], 32, 2, s);
    u1_.init(g_[1], 32, 1, s);
    a_d1_.init(g_[1], 16, 1, s);
    u0_.init(g_[0], 16, 0, s);
    a_d0a_.init(g_[0], 16, 0, s);
    g_out_.init(g_[0], 16, 0, s);
    g_t0_.init(g_[0], 16, 0, s);
    g_u0_.init(g_[0], 16, 0, s);
    g_d1_.init(g_[1], 16, 1, s);
    g_u1_.init(g_[1], 32, 1, s);
    g_d2_.init(g_[2], 32, 2, s);
    g_u2_.init(g_[2], 32, 2, s);
    g_e3b_.init(g_[3], 32, 3, s);
    g_e3a_.init(g_[3], 32, 3, s);
    g_r3_.init(g_[3], 32, 3, s);
    g_e2a_.init(g_[2], 32, 2, s);
    g_r2_.init(g_[2], 32, 2, s);
    g_e1a_.init(g_[1], 32, 1, s);
    g_r1_.init(g_[1], 16, 1, s);
    g_e0a_.init(g_[0], 16, 0, s);
    repack();
    ctx_.sync();
}

void LearnedNet::repack() {
    for (int l = 0; l < kNumLayers; ++l) {
        pack_weights(ctx_, params_.p + woff_[l], wf_[l].p, kLayers[l].cin, kLayers[l].cout, false);
        pack_weights(ctx_, params_.p + woff_[l], wb_[l].p, kLayers[l].cin, kLayers[l].cout, true);
    }
}

void LearnedNet::get_params(float* host) const {
    NUMA_CUDA(cudaMemcpyAsync(host, params_.p, nparams_ * sizeof(float), cudaMemcpyDeviceToHost, ctx_.stream));
    ctx_.sync();
}

void LearnedNet::set_params(const float* host) {
    NUMA_CUDA(cudaMemcpyAsync(params_.p, host, nparams_ * sizeof(float), cudaMemcpyHostToDevice, ctx_.stream));
    repack();
    ctx_.sync();
}

void LearnedNet::conv(int l, const uint4* in, uint4* out, float* o32) {
    const LayerSpec& L = kLayers[l];
    conv3d_tc(ctx_, g_[L.level], L.cin, L.cout, in, reinterpret_cast<const uint4*>(wf_[l].p), params_.p + boff_[l], out,
              o32, L.relu ? 1 : 0, err_.p);
}

void LearnedNet::conv_adj(int l, const uint4* g, uint4* out) {
    const LayerSpec& L = kLayers[l];
    conv3d_tc(ctx_, g_[L.level], L.cout, L.cin, g, reinterpret_cast<const uint4*>(wb_[l].p), nullptr, out, nullptr, 0,
              err_.p);
}

void LearnedNet::dw(int l, const uint4* x, const uint4* g) {
    const LayerSpec& L = kLayers[l];
    conv_dw(ctx_, g_[L.level], L.cin, L.cout, x, g, grad_.p + woff_[l], grad_.p + boff_[l], dw_part_, err_.p);
}

void LearnedNet::forward(const uint4* in, float* out32) {
    conv(E0A, in, a_e0a_.p(), nullptr);
    conv(E0B, a_e0a_.p(), s0_.p(), nullptr);
    planes_restrict(ctx_, s0_.p(), r1_.p(), g_[0], g_[1], 16, 1.0f);
    conv(E1A, r1_.p(), a_e1a_.p(), nullptr);
    conv(E1B, a_e1a_.p(), s1_.p(), nullptr);
    planes_restrict(ctx_, s1_.p(), r2_.p(), g_[1], g_[2], 32, 1.0f);
    conv(E2A, r2_.p(), a_e2a_.p(), nullptr);
    conv(E2B, a_e2a_.p(), s2_.p(), nullptr);
    planes_restrict(ctx_, s2_.p(), r3_.p(), g_[2], g_[3], 32, 1.0f);
    conv(E3A, r3_.p(), a_e3a_.p(), nullptr);
    conv(E3B, a_e3a_.p(), a_e3b_.p(), nullptr);
    planes_prolong(ctx_, a_e3b_.p(), s2_.p(), u2_.p(), g_[3], g_[2], 32, 1.0f, false);
    conv(D2, u2_.p(), a_d2_.p(), nullptr);
    planes_prolong(ctx_, a_d2_.p(), s1_.p(), u1_.p(), g_[2], g_[1], 32, 1.0f, false);
    conv(D1, u1_.p(), a_d1_.p(), nullptr);
    planes_prolong(ctx_, a_d1_.p(), s0_.p(), u0_.p(), g_[1], g_[0], 16, 1.0f, false);
    conv(D0A, u0_.p(), a_d0a_.p(), nullptr);
    conv(D0B, a_d0a_.p(), nullptr, out32);
}

void LearnedNet::zero_grad() { NUMA_CUDA(cudaMemsetAsync(grad_.p, 0, nparams_ * sizeof(float), ctx_.stream)); }

void LearnedNet::loss_and_backward(const uint4* in, const float* t, float* loss_dev) {
    forward(in, out32_.p);
    planes_loss_grad(ctx_, out32_.p, t, g_out_.p(), g_[0], loss_dev);
    dw(D0B, a_d0a_.p(), g_out_.p());
    conv_adj(D0B, g_out_.p(), g_t0_.p());
    planes_relu_mask(ctx_, g_t0_.p(), a_d0a_.p(), g_[0], 16);
    dw(D0A, u0_.p(), g_t0_.p());
    conv_adj(D0A, g_t0_.p(), g_u0_.p());  // gradient of u0 = P d1 + s0: also s0's first part
    planes_restrict(ctx_, g_u0_.p(), g_d1_.p(), g_[0], g_[1], 16, 8.0f);
    planes_relu_mask(ctx_, g_d1_.p(), a_d1_.p(), g_[1], 16);
    dw(D1, u1_.p(), g_d1_.p());
    conv_adj(D1, g_d1_.p(), g_u1_.p());
    planes_restrict(ctx_, g_u1_.p(), g_d2_.p(), g_[1], g_[2], 32, 8.0f);
    planes_relu_mask(ctx_, g_d2_.p(), a_d2_.p(), g_[2], 32);
    dw(D2, u2_.p(), g_d2_.p());
    conv_adj(D2, g_d2_.p(), g_u2_.p());
    planes_restrict(ctx_, g_u2_.p(), g_e3b_.p(), g_[2], g_[3], 32, 8.0f);
    planes_relu_mask(ctx_, g_e3b_.p(), a_e3b_.p(), g_[3], 32);
    dw(E3B, a_e3a_.p(), g_e3b_.p());
    conv_adj(E3B, g_e3b_.p(), g_e3a_.p());
    planes_relu_mask(ctx_, g_e3a_.p(), a_e3a_.p(), g_[3], 32);
    dw(E3A, r3_.p(), g_e3a_.p());
    conv_adj(E3A, g_e3a_.p(), g_r3_.p());
    planes_prolong(ctx_, g_r3_.p(), nullptr, g_u2_.p(), g_[3], g_[2], 32, 0.125f, true);  // s2's gradient
    planes_relu_mask(ctx_, g_u2_.p(), s2_.p(), g_[2], 32);
    dw(E2B, a_e2a_.p(), g_u2_.p());
    conv_adj(E2B, g_u2_.p(), g_e2a_.p());
    planes_relu_mask(ctx_, g_e2a_.p(), a_e2a_.p(), g_[2], 32);
    dw(E2A, r2_.p(), g_e2a_.p());
    conv_adj(E2A, g_e2a_.p(), g_r2_.p());
    planes_prolong(ctx_, g_r2_.p(), nullptr, g_u1_.p(), g_[2], g_[1], 32, 0.125f, true);  // s1's gradient
    planes_relu_mask(ctx_, g_u1_.p(), s1_.p(), g_[1], 32);
    dw(E1B, a_e1a_.p(), g_u1_.p());
    conv_adj(E1B, g_u1_.p(), g_e1a_.p());
    planes_relu_mask(ctx_, g_e1a_.p(), a_e1a_.p(), g_[1], 32);
    dw(E1A, r1_.p(), g_e1a_.p());
    conv_adj(E1A, g_e1a_.p(), g_r1_.p());
    planes_prolong(ctx_, g_r1_.p(), nullptr, g_u0_.p(), g_[1], g_[0], 16, 0.125f, true);  // s0's gradient
    planes_relu_mask(ctx_, g_u0_.p(), s0_.p(), g_[0], 16);
    dw(E0B, a_e0a_.p(), g_u0_.p());
    conv_adj(E0B, g_u0_.p(), g_e0a_.p());
    planes_relu_mask(ctx_, g_e0a_.p(), a_e0a_.p(), g_[0], 16);
    dw(E0A, in, g_e0a_.p());
}

void LearnedNet::adam(float lr) {
    ++step_;
    adam_step(ctx_, params_.p, grad_.p, m_.p, v_.p, nparams_, lr, step_);
    repack();
}

void LearnedNet::check_errors() {
    unsigned h = 0;
    NUMA_CUDA(cudaMemcpyAsync(&h, err_.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx_.stream));
    ctx_.sync();
    if (h) throw Status(NUMA_GPU_ERR_CUDA, "tensor-core convolution: an mbarrier wait gave up");
}

// ------------------------------------------------------------------------------ entry points used by capi.cu
LearnedNet* learned_create(Context& ctx, int n0, uint64_t seed) { return new LearnedNet(ctx, n0, seed); }
void learned_destroy(LearnedNet* net) { delete net; }
size_t learned_num_params(const LearnedNet& net) { return net.num_params(); }
int learned_n0(const LearnedNet& net) { return net.n0(); }
void learned_get_params(const LearnedNet& net, float* host) { net.get_params(host); }
void learned_set_params(LearnedNet& net, const float* host) { net.set_params(host); }

// Host features [n0^3][3] -> output [n0^3] (channel 0).
void learned_forward_host(Context& ctx, LearnedNet& net, const float* feat, float* out) {
    const int n = net.n0();
    const size_t N = (size_t)n * n * n;
    DeviceArray<float> f(3 * N), ones(3);
    std::vector<float> h(3 * N);
    std::memcpy(h.data(), feat, 3 * N * sizeof(float));
    // de-interleave into three FP32 fields
    std::vector<float> r(N), c(N), z(N);
    for (size_t v = 0; v < N; ++v) {
        r[v] = h[3 * v];
        c[v] = h[3 * v + 1];
        z[v] = h[3 * v + 2];
    }
    const float one3[3] = {1.0f, 1.0f, 1.0f};
    NUMA_CUDA(cudaMemcpyAsync(f.p, r.data(), N * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(f.p + N, c.data(), N * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(f.p + 2 * N, z.data(), N * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(ones.p, one3, 3 * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    planes_features(ctx, f.p, f.p + N, f.p + 2 * N, ones.p, net.feature_planes(), net.grid(0));
    net.forward(net.feature_planes(), net.out32());
    std::vector<float> o(N * 16);
    NUMA_CUDA(cudaMemcpyAsync(o.data(), net.out32(), N * 16 * sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    net.check_errors();
    for (size_t v = 0; v < N; ++v) out[v] = o[16 * v];
}

// Host features and target -> loss and the parameter gradient (host, num_params floats).
void learned_grad_host(Context& ctx, LearnedNet& net, const float* feat, const float* target, float* loss,
                       float* grad) {
    const int n = net.n0();
    const size_t N = (size_t)n * n * n;
    DeviceArray<float> f(3 * N), t(N), ones(3), l(1);
    std::vector<float> r(N), c(N), z(N);
    for (size_t v = 0; v < N; ++v) {
        r[v] = feat[3 * v];
        c[v] = feat[3 * v + 1];
        z[v] = feat[3 * v + 2];
    }
    const float one3[3] = {1.0f, 1.0f, 1.0f};
    NUMA_CUDA(cudaMemcpyAsync(f.p, r.data(), N * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(f.p + N, c.data(), N * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(f.p + 2 * N, z.data(), N * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(t.p, target, N * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(ones.p, one3, 3 * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemsetAsync(l.p, 0, sizeof(float), ctx.stream));
    planes_features(ctx, f.p, f.p + N, f.p + 2 * N, ones.p, net.feature_planes(), net.grid(0));
    net.zero_grad();
    net.loss_and_backward(net.feature_planes(), t.p, l.p);
    NUMA_CUDA(cudaMemcpyAsync(loss, l.p, sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(grad, net.grad(), net.num_params() * sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    net.check_errors();
}

// ------------------------------------------------------------------------------ the preconditioner
// Features and correction live on the multigrid level l whose grid is the network's base n0:
// fine n -> (n-1)/2 -> ... -> n0.  Fields are carried between the fine grid and level l by the
// multigrid's full-weighting restriction and trilinear prolongation, FP32, natural layout.
namespace {

__device__ __forceinline__ int split_at_l(int L, int half) { return (L >> 1) + (L & 1) * half; }

// out (nc^3, FP32) = R(f), f the finest FP32 level in the colour-split layout (odd nf)
__global__ void k_rest_from_split(const float* __restrict__ f, float* __restrict__ out, int nf, int half) {
    const int nc = (nf - 1) / 2, Nc = nc * nc * nc;
    const float w[3] = {0.25f, 0.5f, 0.25f};
    const int stride = gridDim.x * blockDim.x;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < Nc; q += stride) {
        const int K = q % nc, J = (q / nc) % nc, I = q / (nc * nc);
        float acc = 0.0f;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                for (int c = 0; c < 3; ++c) {
                    const int L = ((2 * I + a) * nf + (2 * J + b)) * nf + 2 * K + c;
                    acc = __fmaf_rn(w[a] * w[b] * w[c], f[split_at_l(L, half)], acc);
                }
        out[q] = acc;
    }
}

// out (nc^3, FP32) = R(f), f natural (FP64 or FP32)
template <class T>
__global__ void k_rest_nat(const T* __restrict__ f, float* __restrict__ out, int nf) {
    const int nc = (nf - 1) / 2, Nc = nc * nc * nc;
    const float w[3] = {0.25f, 0.5f, 0.25f};
    const int stride = gridDim.x * blockDim.x;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < Nc; q += stride) {
        const int K = q % nc, J = (q / nc) % nc, I = q / (nc * nc);
        float acc = 0.0f;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                for (int c = 0; c < 3; ++c) {
                    const size_t L = ((size_t)(2 * I + a) * nf + (2 * J + b)) * nf + 2 * K + c;
                    acc = __fmaf_rn(w[a] * w[b] * w[c], (float)f[L], acc);
                }
        out[q] = acc;
    }
}

__device__ __forceinline__ float prolong_at(const float* __restrict__ c, int nc, int i, int j, int k) {
    int ci[2], cj[2], ck[2];
    auto terms = [nc](int f, int (&idx)[2]) {
        if (f & 1) {
            idx[0] = (f - 1) >> 1;
            return 1;
        }
        int cnt = 0;
        const int r = f >> 1;
        if (r >= 1) idx[cnt++] = r - 1;
        if (r < nc) idx[cnt++] = r;
        return cnt;
    };
    const int ni = terms(i, ci), nj = terms(j, cj), nk = terms(k, ck);
    const float wt = ((i & 1) ? 1.0f : 0.5f) * ((j & 1) ? 1.0f : 0.5f) * ((k & 1) ? 1.0f : 0.5f);
    float acc = 0.0f;
    for (int a = 0; a < ni; ++a)
        for (int b = 0; b < nj; ++b)
            for (int q = 0; q < nk; ++q) acc = __fmaf_rn(wt, c[((size_t)ci[a] * nc + cj[b]) * nc + ck[q]], acc);
    return acc;
}

// f (nf^3 = (2 nc + 1)^3, FP32) = P(c)
__global__ void k_prolong_nat(const float* __restrict__ c, float* __restrict__ f, int nc) {
    const int nf = 2 * nc + 1, Nf = nf * nf * nf;
    const int stride = gridDim.x * blockDim.x;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < Nf; p += stride)
        f[p] = prolong_at(c, nc, p / (nf * nf), (p / nf) % nf, p % nf);
}

// z (fine FP64) += s * P(c), s a device scalar
__global__ void k_prolong_add_fine(const float* __restrict__ c, double* __restrict__ z, int nc,
                                   const float* __restrict__ s) {
    const int nf = 2 * nc + 1;
    const size_t Nf = (size_t)nf * nf * nf;
    const float sc = *s;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < Nf; p += stride) {
        const int i = (int)(p / ((size_t)nf * nf)), j = (int)((p / nf) % nf), k = (int)(p % nf);
        z[p] = z[p] + f32_to_f64(sc * prolong_at(c, nc, i, j, k));
    }
}

// s = max(sqrt(mean a^2), tiny); scales = {1/s, 1/10, 0} (one block)
__global__ void k_rms_scales(const float* __restrict__ a, int N, float* __restrict__ s, float* __restrict__ scales) {
    __shared__ float sm[32];
    float acc = 0.0f;
    for (int i = threadIdx.x; i < N; i += blockDim.x) acc = __fmaf_rn(a[i], a[i], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
        const float r = fmaxf(sqrtf(t / (float)N), 1e-30f);
        *s = r;
        scales[0] = 1.0f / r;
        scales[1] = 0.1f;
        scales[2] = 0.0f;
    }
}

// out[v] = y32[16 v] (channel 0 of the network output)
__global__ void k_channel0(const float* __restrict__ y32, float* __restrict__ out, int N) {
    const int stride = gridDim.x * blockDim.x;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += stride) out[v] = y32[(size_t)16 * v];
}

// r = sum of 8 Gaussian bumps: params [8][5] = (cx, cy, cz, width, amplitude) on the unit cube
__global__ void k_bumps(double* __restrict__ r, int n, const float* __restrict__ bp) {
    const size_t N = (size_t)n * n * n;
    const float h = 1.0f / (float)(n + 1);
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) {
        const float x = (float)(p % n + 1) * h, y = (float)((p / n) % n + 1) * h, z = (float)(p / ((size_t)n * n) + 1) * h;
        float acc = 0.0f;
        for (int b = 0; b < 8; ++b) {
            const float dx = x - bp[5 * b], dy = y - bp[5 * b + 1], dz = z - bp[5 * b + 2], w = bp[5 * b + 3];
            acc += bp[5 * b + 4] * expf(-(dx * dx + dy * dy + dz * dz) / (2.0f * w * w));
        }
        r[p] = (double)acc;
    }
}

__global__ void k_axpby64(const double* __restrict__ a, double alpha, const double* __restrict__ b, double beta,
                          double* __restrict__ out, size_t N) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) out[p] = alpha * a[p] + beta * b[p];
}

// t = x / s (device scalar)
__global__ void k_div_scalar(const float* __restrict__ x, const float* __restrict__ s, float* __restrict__ t, int N) {
    const float inv = 1.0f / *s;
    const int stride = gridDim.x * blockDim.x;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += stride) t[v] = x[v] * inv;
}

unsigned ew(const Context& ctx, size_t N) {
    return (unsigned)std::max<size_t>(1, std::min<size_t>((N + 255) / 256, (size_t)ctx.sm_count * 16));
}

}  // namespace

// The restriction / prolongation chains between a fine grid and the network's level.
class LevelChain {
public:
    LevelChain(Context& ctx, int n_fine, int n0) : ctx_(ctx) {
        int n = n_fine;
        ns_.push_back(n);
        while (n > n0) {
            if (!(n & 1)) break;
            n = (n - 1) / 2;
            ns_.push_back(n);
        }
        if (n != n0 || ns_.size() < 2)
            throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT,
                         "learned preconditioner: the fine grid must coarsen to the network's base grid");
        for (size_t l = 1; l < ns_.size(); ++l) {
            const size_t Nl = (size_t)ns_[l] * ns_[l] * ns_[l];
            a_.emplace_back(Nl);
            b_.emplace_back(Nl);
        }
    }
    int levels() const { return (int)ns_.size() - 1; }
    int n_at(int l) const { return ns_[l]; }
    size_t N0() const { return (size_t)ns_.back() * ns_.back() * ns_.back(); }
    // out (base grid, FP32) = R^l f; the first step reads the fine array (split FP32, or natural T)
    const float* restrict_split(const float* f_split, float* out) {
        const int nf = ns_[0];
        const int half = (int)(((size_t)nf * nf * nf + 1) / 2);
        float* cur = levels() == 1 ? out : a_[0].p;
        k_rest_from_split<<<ew(ctx_, a_[0].n), 256, 0, ctx_.stream>>>(f_split, cur, nf, half);
        ctx_.count_launch();
        return chain(cur, out);
    }
    template <class T>
    const float* restrict_nat(const T* f, float* out) {
        float* cur = levels() == 1 ? out : a_[0].p;
        k_rest_nat<T><<<ew(ctx_, a_[0].n), 256, 0, ctx_.stream>>>(f, cur, ns_[0]);
        ctx_.count_launch();
        return chain(cur, out);
    }
    // z (fine FP64) += s * P^l d (d on the base grid)
    void prolong_add(const float* d, double* z, const float* s) {
        const float* cur = d;
        for (int l = levels(); l > 1; --l) {
            float* nxt = b_[l - 2].p;  // level l-1
            k_prolong_nat<<<ew(ctx_, b_[l - 2].n), 256, 0, ctx_.stream>>>(cur, nxt, ns_[l]);
            ctx_.count_launch();
            cur = nxt;
        }
        k_prolong_add_fine<<<ew(ctx_, (size_t)ns_[0] * ns_[0] * ns_[0]), 256, 0, ctx_.stream>>>(cur, z, ns_[1], s);
        ctx_.count_launch();
    }

private:
    const float* chain(float* cur, float* out) {
        for (int l = 1; l < levels(); ++l) {
            float* nxt = (l + 1 == levels()) ? out : a_[l].p;
            k_rest_nat<float><<<ew(ctx_, (size_t)ns_[l + 1] * ns_[l + 1] * ns_[l + 1]), 256, 0, ctx_.stream>>>(cur, nxt,
                                                                                                          ns_[l]);
            ctx_.count_launch();
            cur = nxt;
        }
        return out;
    }
    Context& ctx_;
    std::vector<int> ns_;
    std::vector<DeviceArray<float>> a_, b_;
};

// z = V(r) + s P^l net(R^l q / s, R^l c / 10) with q = r - J V(r) the residual the V-cycle leaves and
// s = rms(R^l q): the network stands in for the coarse solve of the error equation J e = q, which
// the Poisson V-cycle (built for -Laplacian alone) does not see the -c term of.  FGMRES's
// preconditioner; the plain V-cycle serves the rest of a linear solve once the residual reduction
// per iteration stalls.
class LearnedProvider : public Provider {
public:
    LearnedProvider(Context& ctx, size_t n, LearnedNet& net, double stall)
        : ctx_(ctx), mg_(ctx, n, 2, 2, NUMA_GPU_FP32, 0), net_(net), chain_(ctx, (int)n, net.n0()), stall_(stall),
          n_((int)n), h2inv_((n + 1.0) * (n + 1.0)) {
        const size_t N0 = chain_.N0(), N = n * n * n;
        c32_.resize(N);
        w_.resize(N);
        r0_.resize(N0);
        c0_.resize(N0);
        d0_.resize(N0);
        s_.resize(4);
        NUMA_CUDA(cudaMemsetAsync(c0_.p, 0, N0 * sizeof(float), ctx_.stream));
    }
    void make(const double* x, const double* cache) override {
        (void)x;
        if (cache) {
            chain_.restrict_nat<double>(cache, c0_.p);
            bratu_coef32(ctx_, cache, c32_.p, c32_.n);
        } else {
            NUMA_CUDA(cudaMemsetAsync(c0_.p, 0, c0_.n * sizeof(float), ctx_.stream));
            NUMA_CUDA(cudaMemsetAsync(c32_.p, 0, c32_.n * sizeof(float), ctx_.stream));
        }
        use_net_ = true;
        prev_ = 1.0;
    }
    void apply(const double* r, double* z) override {
        mg_.apply(r, z);
        if (!use_net_) return;
        const int N0 = (int)chain_.N0();
        // q = r - J z, restricted
        bratu_jvp32(ctx_, n_, h2inv_, c32_.p, z, w_.p);
        k_axpby64<<<ew(ctx_, w_.n), 256, 0, ctx_.stream>>>(r, 1.0, w_.p, -1.0, w_.p, w_.n);
        ctx_.count_launch();
        chain_.restrict_nat<double>(w_.p, r0_.p);
        k_rms_scales<<<1, 512, 0, ctx_.stream>>>(r0_.p, N0, s_.p, s_.p + 1);
        ctx_.count_launch();
        planes_features(ctx_, r0_.p, c0_.p, r0_.p, s_.p + 1, net_.feature_planes(), net_.grid(0));
        net_.forward(net_.feature_planes(), net_.out32());
        k_channel0<<<ew(ctx_, N0), 256, 0, ctx_.stream>>>(net_.out32(), d0_.p, N0);
        ctx_.count_launch();
        chain_.prolong_add(d0_.p, z, s_.p);
        ++net_applies_;
    }
    void progress(size_t iters, double rel_res) override {
        if (iters <= 1) prev_ = 1.0;
        if (use_net_ && iters >= 2 && rel_res > stall_ * prev_) {
            use_net_ = false;
            ++fallbacks_;
        }
        prev_ = rel_res;
    }
    int kind() const override { return NUMA_GPU_PRECOND_LEARNED; }
    size_t net_applies() const { return net_applies_; }
    size_t fallbacks() const { return fallbacks_; }

private:
    Context& ctx_;
    PoissonMG mg_;
    LearnedNet& net_;
    LevelChain chain_;
    double stall_;
    int n_;
    double h2inv_;
    DeviceArray<float> r0_, c0_, d0_, s_, c32_;
    DeviceArray<double> w_;
    bool use_net_ = true;
    double prev_ = 1.0;
    size_t net_applies_ = 0, fallbacks_ = 0;
};

std::unique_ptr<Provider> make_learned_provider(Context& ctx, size_t n, LearnedNet& net, double stall) {
    return std::make_unique<LearnedProvider>(ctx, n, net, stall);
}

void learned_provider_stats(Provider& p, size_t* applies, size_t* fallbacks) {
    auto* lp = dynamic_cast<LearnedProvider*>(&p);
    if (!lp) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "not a learned preconditioner");
    *applies = lp->net_applies();
    *fallbacks = lp->fallbacks();
}

// ------------------------------------------------------------------------------ training
namespace {
// J e = r at a Bratu3D iterate with coefficient c (FP64 analytic product)
struct CoefJacobian : LinearOp {
    Bratu3D& f;
    const double* c;
    CoefJacobian(Bratu3D& op, const double* cc) : f(op), c(cc) {}
    void apply(const double* v, double* out) override { f.jvp_c(c, v, out); }
};
struct MGPre : Precond {
    PoissonMG& mg;
    explicit MGPre(PoissonMG& m) : mg(m) {}
    void apply(const double* r, double* z) override { mg.apply(r, z); }
};
}  // namespace

void learned_train(Context& ctx, LearnedNet& net, const numa_learned_train_params& p, numa_learned_train_report& rep) {
    std::memset(&rep, 0, sizeof(rep));
    const int n = (int)p.n_fine;
    const size_t N = (size_t)n * n * n;
    LevelChain chain(ctx, n, net.n0());
    const size_t N0 = chain.N0();
    const int per_state = 1 + p.krylov_per_state + p.rhs_per_state;
    const size_t samples = (size_t)p.instances * p.states * per_state;
    if (samples == 0) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "no training samples requested");
    DeviceArray<float> feats(samples * 2 * N0), targets(samples * N0);
    DeviceArray<double> u(N), us(N), c(N), F(N), r(N), e(N), zmg(N), diff(N), qres(N);
    DeviceArray<float> c32(N);
    const double h2inv = (n + 1.0) * (n + 1.0);
    DeviceArray<float> tmp(N0), sc(4), bp(40);
    PoissonMG mg(ctx, (size_t)n, 2, 2, NUMA_GPU_FP32, 0);
    Gmres gm(ctx, N);
    std::mt19937_64 rng(p.seed);
    std::uniform_real_distribution<double> U01(0.0, 1.0);
    const auto t0 = std::chrono::steady_clock::now();
    size_t k = 0;
    for (int inst = 0; inst < p.instances; ++inst) {
        const double lam = p.lambda_min + (p.lambda_max - p.lambda_min) * U01(rng);
        Bratu3D op(ctx, (size_t)n, lam);
        // u* by the mixed Newton-Krylov solve
        NUMA_CUDA(cudaMemsetAsync(u.p, 0, N * sizeof(double), ctx.stream));
        {
            KrylovParams kp;
            kp.rtol_nl = 1e-8;
            kp.restart = 30;
            kp.flexible = true;
            kp.jvp_precision = NUMA_GPU_FP32;
            auto pc = make_mg_provider(ctx, (size_t)n, 2, 2, NUMA_GPU_FP32, 0);
            numa_krylov_result res;
            newton_krylov(op, u.p, kp, pc.get(), res);
        }
        for (int st = 0; st < p.states; ++st) {
            const double sfac = p.states == 1 ? 1.0 : (double)st / (double)(p.states - 1);
            k_axpby64<<<ew(ctx, N), 256, 0, ctx.stream>>>(u.p, sfac, u.p, 0.0, us.p, N);
            ctx.count_launch();
            // c holds N doubles: the FP64 cache (the mixed solve above left the operator keeping
            // RN32(c) and RN32(F) after them, which would write past c)
            op.prepare_cache(NUMA_GPU_FP64);
            op.eval(us.p, F.p, c.p, nullptr);
            const float* c0 = chain.restrict_nat<double>(c.p, tmp.p);
            bratu_coef32(ctx, c.p, c32.p, N);
            // r = a seeded sum of 8 Gaussian bumps (centres in the cube, widths 0.05..0.2, amplitudes +-1)
            auto bumps = [&]() {
                float h[40];
                for (int b = 0; b < 8; ++b) {
                    h[5 * b] = (float)U01(rng);
                    h[5 * b + 1] = (float)U01(rng);
                    h[5 * b + 2] = (float)U01(rng);
                    h[5 * b + 3] = (float)(0.05 + 0.15 * U01(rng));
                    h[5 * b + 4] = (float)(2.0 * U01(rng) - 1.0);
                }
                NUMA_CUDA(cudaMemcpyAsync(bp.p, h, sizeof(h), cudaMemcpyHostToDevice, ctx.stream));
                k_bumps<<<ew(ctx, N), 256, 0, ctx.stream>>>(r.p, n, bp.p);
                ctx.count_launch();
            };
            KrylovSpace space;
            size_t kry = 0;  // Arnoldi vectors available from the F(u) solve
            for (int q = 0; q < per_state; ++q) {
                if (q == 0) {
                    dev_copy(ctx, F.p, r.p, N);
                } else if (q <= p.krylov_per_state && (size_t)q <= kry) {
                    dev_copy(ctx, space.V.p + (size_t)q * N, r.p, N);  // V_q of the F(u) solve
                } else {
                    bumps();  // (also when the F(u) solve stopped before V_q)
                }
                // e = J^-1 r (GMG-preconditioned FGMRES), z = V(r)
                CoefJacobian J(op, c.p);
                MGPre M(mg);
                GmresOptions o;
                o.rtol = p.solve_rtol;
                o.restart = 30;
                o.max_iters = 300;
                o.flexible = true;
                if (q == 0) {
                    space.clear();
                    gm.solve(J, &M, r.p, e.p, o, &space);
                    kry = space.k;
                } else {
                    gm.solve(J, &M, r.p, e.p, o);
                }
                mg.apply(r.p, zmg.p);
                // the residual the V-cycle leaves, q = r - J z (the provider's FP32 product)
                bratu_jvp32(ctx, n, h2inv, c32.p, zmg.p, qres.p);
                k_axpby64<<<ew(ctx, N), 256, 0, ctx.stream>>>(r.p, 1.0, qres.p, -1.0, qres.p, N);
                ctx.count_launch();
                float* fr = feats.p + k * 2 * N0;
                float* fc = fr + N0;
                chain.restrict_nat<double>(qres.p, fr);
                k_rms_scales<<<1, 512, 0, ctx.stream>>>(fr, (int)N0, sc.p, sc.p + 1);
                ctx.count_launch();
                k_div_scalar<<<ew(ctx, N0), 256, 0, ctx.stream>>>(fr, sc.p, fr, (int)N0);
                ctx.count_launch();
                // coefficient feature (scaled by 1/10 when the planes are formed)
                NUMA_CUDA(cudaMemcpyAsync(fc, c0, N0 * sizeof(float), cudaMemcpyDeviceToDevice, ctx.stream));
                // target = R^l (e - z) / s
                k_axpby64<<<ew(ctx, N), 256, 0, ctx.stream>>>(e.p, 1.0, zmg.p, -1.0, diff.p, N);
                ctx.count_launch();
                float* tt = targets.p + k * N0;
                chain.restrict_nat<double>(diff.p, tt);
                k_div_scalar<<<ew(ctx, N0), 256, 0, ctx.stream>>>(tt, sc.p, tt, (int)N0);
                ctx.count_launch();
                ++k;
            }
        }
        ctx.check_launch("learned training data");
    }
    ctx.sync();
    rep.samples = k;
    rep.gen_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    {
        std::vector<float> th(k * N0);
        NUMA_CUDA(cudaMemcpyAsync(th.data(), targets.p, th.size() * sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
        ctx.sync();
        double acc = 0.0;
        for (float v : th) acc += (double)v * v;
        rep.target_ms = (float)(acc / (double)th.size());
    }
    // training: Adam over shuffled samples, gradients summed over a batch
    const auto t1 = std::chrono::steady_clock::now();
    std::vector<size_t> order(k);
    for (size_t i = 0; i < k; ++i) order[i] = i;
    DeviceArray<float> loss(1), scales(4);
    const float sc_h[4] = {1.0f, 0.1f, 0.0f, 0.0f};
    NUMA_CUDA(cudaMemcpyAsync(scales.p, sc_h, sizeof(sc_h), cudaMemcpyHostToDevice, ctx.stream));
    const int batch = std::max(1, p.batch);
    for (int ep = 0; ep < p.epochs; ++ep) {
        std::shuffle(order.begin(), order.end(), rng);
        NUMA_CUDA(cudaMemsetAsync(loss.p, 0, sizeof(float), ctx.stream));
        for (size_t i = 0; i < k; i += batch) {
            net.zero_grad();
            for (size_t b = i; b < std::min(k, i + batch); ++b) {
                const float* fr = feats.p + order[b] * 2 * N0;
                planes_features(ctx, fr, fr + N0, fr, scales.p, net.feature_planes(), net.grid(0));
                net.loss_and_backward(net.feature_planes(), targets.p + order[b] * N0, loss.p);
            }
            net.adam(p.lr);
        }
        float lh = 0.0f;
        NUMA_CUDA(cudaMemcpyAsync(&lh, loss.p, sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
        ctx.sync();
        lh /= (float)k;
        if (ep == 0) rep.loss_first = lh;
        rep.loss_last = lh;
    }
    net.check_errors();
    rep.train_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
}

}  // namespace numa::gpu
