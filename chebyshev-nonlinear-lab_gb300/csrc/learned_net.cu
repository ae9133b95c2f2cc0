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
void conv_dw(Context& ctx, const VoxGrid& gr, int cin, int cout, const uint4* x, const uint4* g, float* dw, float* db);
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
    conv_dw(ctx_, g_[L.level], L.cin, L.cout, x, g, grad_.p + woff_[l], grad_.p + boff_[l]);
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

}  // namespace numa::gpu
