// learned.cu — the learned preconditioner's building blocks: packing between FP32 channel-last
// arrays and the BF16 8-channel plane layout, and the launch of the tensor-core convolution
// (learned_conv.cuh) for every supported channel pair.
#include <algorithm>
#include <cmath>
#include <vector>

#include "learned_conv.cuh"
#include "numa_internal.hpp"

namespace numa::gpu {
namespace {

// FP32 channel-last x[v][C] (v = (z n + y) n + x) -> BF16 planes (interior rows; halo untouched).
__global__ void k_pack_act(const float* __restrict__ x, uint4* __restrict__ planes, VoxGrid g, int C) {
    const int N = g.n * g.n * g.n, P8 = C / 8;
    const int stride = gridDim.x * blockDim.x;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N * P8; e += stride) {
        const int v = e / P8, p = e - v * P8;
        const int xx = v % g.n, yy = (v / g.n) % g.n, zz = v / (g.n * g.n);
        const float* s = x + (size_t)v * C + 8 * p;
        uint4 pk;
        pk.x = pack_bf16x2(s[0], s[1]);
        pk.y = pack_bf16x2(s[2], s[3]);
        pk.z = pack_bf16x2(s[4], s[5]);
        pk.w = pack_bf16x2(s[6], s[7]);
        const int q = ((zz + 1) * g.np + (yy + 1)) * g.np + (xx + 1);
        planes[(size_t)p * g.rows + g.front + q] = pk;
    }
}

// FP32 weights W[tap][ci][co] -> BF16 B operand [tap][k16 chunk][half][co_out][8] of the layer
// with CIN' = cin, COUT' = cout; FLIP: the weights of the adjoint convolution (gradient with respect
// to the input): W'[tap][co][ci] = W[26 - tap][ci][co], i.e. CIN' = cout, COUT' = cin.
__global__ void k_pack_w(const float* __restrict__ w, __nv_bfloat16* __restrict__ wg, int cin, int cout, int flip) {
    const int ci_n = flip ? cout : cin, co_n = flip ? cin : cout;  // the packed layer's CIN', COUT'
    const int total = 27 * ci_n * co_n;
    const int stride = gridDim.x * blockDim.x;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
        // e enumerates the packed layout: [tap][kc][half][co'][8]
        const int k8 = e % 8, rest = e / 8;
        const int co = rest % co_n, rest2 = rest / co_n;
        const int h = rest2 % 2, rest3 = rest2 / 2;
        const int kc = rest3 % (ci_n / 16), tap = rest3 / (ci_n / 16);
        const int ci = kc * 16 + h * 8 + k8;
        const float val = flip ? w[((size_t)(26 - tap) * cin + co) * cout + ci] : w[((size_t)tap * cin + ci) * cout + co];
        wg[e] = __float2bfloat16_rn(val);
    }
}

template <int CIN, int COUT, bool OUT32, int NST>
void launch_conv_stages(Context& ctx, const VoxGrid& g, const uint4* in, const uint4* wg, const float* bias, uint4* out,
                        float* out32, int relu, unsigned* err, size_t smem) {
    // persistent CTAs: as many as fit on the GPU at once, each pipelining its tiles
    int per_sm = 0;
    NUMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv3d_tc<CIN, COUT, OUT32, NST>, kConvThreads,
                                                            smem));
    const int grid = std::max(1, std::min(g.tiles, std::max(1, per_sm) * ctx.sm_count));
    k_conv3d_tc<CIN, COUT, OUT32, NST><<<grid, kConvThreads, smem, ctx.stream>>>(in, wg, bias, out, out32, g, relu, err);
    ctx.count_launch();
}

// Three span buffers where they fit in shared memory, else two.
template <int CIN, int COUT, bool OUT32>
void launch_conv(Context& ctx, const VoxGrid& g, const uint4* in, const uint4* wg, const float* bias, uint4* out,
                 float* out32, int relu, unsigned* err) {
    if (OUT32 && (reinterpret_cast<uintptr_t>(out32) & 15u))
        throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "convolution FP32 output must be 16-byte aligned");
    const int lim3 = set_dynamic_smem_limit(ctx, k_conv3d_tc<CIN, COUT, OUT32, 3>);
    const int lim2 = set_dynamic_smem_limit(ctx, k_conv3d_tc<CIN, COUT, OUT32, 2>);
    const size_t s3 = conv_smem_bytes<CIN, COUT>(g, 3), s2 = conv_smem_bytes<CIN, COUT>(g, 2);
    if (s3 <= (size_t)lim3) launch_conv_stages<CIN, COUT, OUT32, 3>(ctx, g, in, wg, bias, out, out32, relu, err, s3);
    else if (s2 <= (size_t)lim2) launch_conv_stages<CIN, COUT, OUT32, 2>(ctx, g, in, wg, bias, out, out32, relu, err, s2);
    else throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "convolution tile exceeds shared memory");
}

__device__ __forceinline__ void unpack8(const uint4 u, float (&f)[8]) {
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        f[2 * i] = __uint_as_float(w[i] << 16);
        f[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
    }
}
__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
    uint4 u;
    u.x = pack_bf16x2(f[0], f[1]);
    u.y = pack_bf16x2(f[2], f[3]);
    u.z = pack_bf16x2(f[4], f[5]);
    u.w = pack_bf16x2(f[6], f[7]);
    return u;
}
__device__ __forceinline__ size_t prow(const VoxGrid& g, int p, int x, int y, int z) {
    return (size_t)p * g.rows + g.front + ((size_t)(z + 1) * g.np + (y + 1)) * g.np + (x + 1);
}

// coarse = scale * R(fine) per channel: the 27-point full weighting of the multigrid restriction
// (weights (1/4, 1/2, 1/4) per dimension, summed a (z) outer, b (y), c (x) inner), FP32.
__global__ void k_restrict_planes(const uint4* __restrict__ fine, uint4* __restrict__ coarse, VoxGrid gf, VoxGrid gc,
                                  int P8, float scale) {
    const int Nc = gc.n * gc.n * gc.n;
    const int stride = gridDim.x * blockDim.x;
    const float w[3] = {0.25f, 0.5f, 0.25f};
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < Nc * P8; e += stride) {
        const int v = e % Nc, p = e / Nc;
        const int K = v % gc.n, J = (v / gc.n) % gc.n, I = v / (gc.n * gc.n);
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                for (int c = 0; c < 3; ++c) {
                    float f[8];
                    unpack8(fine[prow(gf, p, 2 * K + c, 2 * J + b, 2 * I + a)], f);
                    const float wt = w[a] * w[b] * w[c];
#pragma unroll
                    for (int i = 0; i < 8; ++i) acc[i] = __fmaf_rn(wt, f[i], acc[i]);
                }
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i] = acc[i] * scale;
        coarse[prow(gc, p, K, J, I)] = pack8(acc);
    }
}

__device__ __forceinline__ int interp1(int f, int nc, int (&idx)[2]) {
    if (f & 1) {
        idx[0] = (f - 1) >> 1;
        return 1;
    }
    int cnt = 0;
    const int right = f >> 1;
    if (right >= 1) idx[cnt++] = right - 1;
    if (right < nc) idx[cnt++] = right;
    return cnt;
}

// out = [out +] [add +] scale * P(coarse) per channel: the trilinear interpolation of the
// multigrid prolongation (weight 1 at an odd fine index, 1/2 per neighbour at an even one), FP32.
__global__ void k_prolong_planes(const uint4* __restrict__ coarse, const uint4* __restrict__ add, uint4* out,
                                 VoxGrid gc, VoxGrid gf, int P8, float scale, int accumulate) {
    const int Nf = gf.n * gf.n * gf.n;
    const int stride = gridDim.x * blockDim.x;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < Nf * P8; e += stride) {
        const int v = e % Nf, p = e / Nf;
        const int k = v % gf.n, j = (v / gf.n) % gf.n, i = v / (gf.n * gf.n);
        int ci[2], cj[2], ck[2];
        const int ni = interp1(i, gc.n, ci), nj = interp1(j, gc.n, cj), nk = interp1(k, gc.n, ck);
        const float wt = ((i & 1) ? 1.0f : 0.5f) * ((j & 1) ? 1.0f : 0.5f) * ((k & 1) ? 1.0f : 0.5f);
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int a = 0; a < ni; ++a)
            for (int b = 0; b < nj; ++b)
                for (int c = 0; c < nk; ++c) {
                    float f[8];
                    unpack8(coarse[prow(gc, p, ck[c], cj[b], ci[a])], f);
#pragma unroll
                    for (int q = 0; q < 8; ++q) acc[q] = __fmaf_rn(wt, f[q], acc[q]);
                }
        const size_t o = prow(gf, p, k, j, i);
        float r[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) r[q] = acc[q] * scale;
        if (add) {
            float f[8];
            unpack8(add[o], f);
#pragma unroll
            for (int q = 0; q < 8; ++q) r[q] = f[q] + r[q];
        }
        if (accumulate) {
            float f[8];
            unpack8(out[o], f);
#pragma unroll
            for (int q = 0; q < 8; ++q) r[q] = f[q] + r[q];
        }
        out[o] = pack8(r);
    }
}

// g = y > 0 ? g : 0 (gradient through a ReLU whose output is y), interior voxels.
__global__ void k_relu_mask_planes(uint4* __restrict__ g, const uint4* __restrict__ y, VoxGrid gr, int P8) {
    const int N = gr.n * gr.n * gr.n;
    const int stride = gridDim.x * blockDim.x;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N * P8; e += stride) {
        const int v = e % N, p = e / N;
        const size_t o = prow(gr, p, v % gr.n, (v / gr.n) % gr.n, v / (gr.n * gr.n));
        float a[8], b[8];
        unpack8(g[o], a);
        unpack8(y[o], b);
#pragma unroll
        for (int q = 0; q < 8; ++q) a[q] = b[q] > 0.0f ? a[q] : 0.0f;
        g[o] = pack8(a);
    }
}

// dw[e] += sum over the CTAs c of part[c][e], in CTA order (the tensor-core weight gradient's partials)
__global__ void k_dw_reduce(const float* __restrict__ part, int nparts, int count, float* __restrict__ dw) {
    const int stride = gridDim.x * blockDim.x;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += stride) {
        float s = 0.0f;
        for (int c = 0; c < nparts; ++c) s += part[(size_t)c * count + e];
        dw[e] += s;
    }
}

// db[co] += sum over the interior voxels of g[v][co]: one block per output channel, FP32 sums per
// thread, the block's total in FP64 (deterministic).
__global__ void __launch_bounds__(256) k_bias_grad(const uint4* __restrict__ g, VoxGrid gr, float* __restrict__ db) {
    const int co = blockIdx.x, pl = co / 8, q = co % 8;
    const int N = gr.n * gr.n * gr.n;
    float s = 0.0f;
    for (int v = threadIdx.x; v < N; v += 256) {
        const int xx = v % gr.n, yy = (v / gr.n) % gr.n, zz = v / (gr.n * gr.n);
        float f[8];
        unpack8(g[prow(gr, pl, xx, yy, zz)], f);
        s += f[q];
    }
    double acc[1] = {(double)s};
    __shared__ double sm[1][32];
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) db[co] += (float)acc[0];
}

// 16-channel feature planes: channel 0 = sr r, 1 = sc c, 2 = sz z, 3..15 = 0 (FP32 natural in).
__global__ void k_feat_planes(const float* __restrict__ r, const float* __restrict__ c, const float* __restrict__ z,
                              const float* __restrict__ scales, uint4* __restrict__ planes, VoxGrid gr) {
    const int N = gr.n * gr.n * gr.n;
    const int stride = gridDim.x * blockDim.x;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += stride) {
        float f[8] = {r[v] * scales[0], c[v] * scales[1], z[v] * scales[2], 0, 0, 0, 0, 0};
        const float zero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const int xx = v % gr.n, yy = (v / gr.n) % gr.n, zz = v / (gr.n * gr.n);
        planes[prow(gr, 0, xx, yy, zz)] = pack8(f);
        planes[prow(gr, 1, xx, yy, zz)] = pack8(zero8);
    }
}

// Loss of the network output (channel 0 of y32 [N][16]) against t: g (16-channel planes) =
// (2 / N)(y0 - t) in channel 0, zero elsewhere; *loss += sum (y0 - t)^2 / N.
__global__ void k_loss_grad(const float* __restrict__ y32, const float* __restrict__ t, uint4* __restrict__ g,
                            VoxGrid gr, float* __restrict__ loss) {
    const int N = gr.n * gr.n * gr.n;
    const int stride = gridDim.x * blockDim.x;
    float part = 0.0f;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += stride) {
        const float d = y32[(size_t)v * 16] - t[v];
        part = __fmaf_rn(d, d, part);
        float f[8] = {2.0f * d / (float)N, 0, 0, 0, 0, 0, 0, 0};
        const float zero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const int xx = v % gr.n, yy = (v / gr.n) % gr.n, zz = v / (gr.n * gr.n);
        g[prow(gr, 0, xx, yy, zz)] = pack8(f);
        g[prow(gr, 1, xx, yy, zz)] = pack8(zero8);
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, part / (float)N);
}

// Adam (Kingma and Ba, 2015) on FP32 master parameters.
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       size_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

}  // namespace

// Dispatches k_conv3d_tc over the supported channel pairs.
void conv3d_tc(Context& ctx, const VoxGrid& g, int cin, int cout, const uint4* in, const uint4* wg,
               const float* bias, uint4* out, float* out32, int relu, unsigned* err) {
    if (g.n > 63) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "tensor-core convolution: grid above 63^3");
    const bool o32 = out32 != nullptr;
#define NUMA_CONV_CASE(CI, CO)                                                              \
    if (cin == CI && cout == CO) {                                                          \
        if (o32) launch_conv<CI, CO, true>(ctx, g, in, wg, bias, out, out32, relu, err);    \
        else launch_conv<CI, CO, false>(ctx, g, in, wg, bias, out, out32, relu, err);       \
        ctx.check_launch("conv3d_tc");                                                      \
        return;                                                                             \
    }
    NUMA_CONV_CASE(16, 16)
    NUMA_CONV_CASE(16, 32)
    NUMA_CONV_CASE(32, 16)
    NUMA_CONV_CASE(32, 32)
#undef NUMA_CONV_CASE
    throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "tensor-core convolution: channel counts must be 16 or 32");
}

namespace {
unsigned grid_for(const Context& ctx, size_t work) {
    return (unsigned)std::max<size_t>(1, std::min<size_t>((work + 255) / 256, (size_t)ctx.sm_count * 16));
}
}  // namespace

void planes_restrict(Context& ctx, const uint4* fine, uint4* coarse, const VoxGrid& gf, const VoxGrid& gc, int C,
                     float scale) {
    k_restrict_planes<<<grid_for(ctx, (size_t)gc.n * gc.n * gc.n * (C / 8)), 256, 0, ctx.stream>>>(fine, coarse, gf, gc,
                                                                                                 C / 8, scale);
    ctx.count_launch();
}

void planes_prolong(Context& ctx, const uint4* coarse, const uint4* add, uint4* out, const VoxGrid& gc,
                    const VoxGrid& gf, int C, float scale, bool accumulate) {
    k_prolong_planes<<<grid_for(ctx, (size_t)gf.n * gf.n * gf.n * (C / 8)), 256, 0, ctx.stream>>>(
        coarse, add, out, gc, gf, C / 8, scale, accumulate ? 1 : 0);
    ctx.count_launch();
}

void planes_relu_mask(Context& ctx, uint4* g, const uint4* y, const VoxGrid& gr, int C) {
    k_relu_mask_planes<<<grid_for(ctx, (size_t)gr.n * gr.n * gr.n * (C / 8)), 256, 0, ctx.stream>>>(g, y, gr, C / 8);
    ctx.count_launch();
}

template <int CIN, int COUT>
void launch_conv_dw(Context& ctx, const VoxGrid& gr, const uint4* x, const uint4* g, float* dw, float* db,
                    DeviceArray<float>& part, unsigned* err) {
    const size_t smem = dw_smem_bytes<CIN, COUT>(gr);
    const int lim = set_dynamic_smem_limit(ctx, k_conv_dw_tc<CIN, COUT>);
    if (smem > (size_t)lim) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "weight-gradient tile exceeds shared memory");
    // one CTA per SM at most (512 tensor-memory columns at C_out = 32), each accumulating its tiles
    const int grid = std::max(1, std::min(gr.tiles, ctx.sm_count));
    const int count = 27 * CIN * COUT;
    part.resize((size_t)grid * count);
    k_conv_dw_tc<CIN, COUT><<<grid, 128, smem, ctx.stream>>>(x, g, gr, part.p, err);
    k_dw_reduce<<<(count + 255) / 256, 256, 0, ctx.stream>>>(part.p, grid, count, dw);
    k_bias_grad<<<COUT, 256, 0, ctx.stream>>>(g, gr, db);
    ctx.count_launch(3);
}

// dW += the weight gradient (BF16 operands on the tensor cores, FP32 accumulation), db += the bias
// gradient; part is the caller's scratch for the per-CTA partials, err the mbarrier give-up flag.
void conv_dw(Context& ctx, const VoxGrid& gr, int cin, int cout, const uint4* x, const uint4* g, float* dw, float* db,
             DeviceArray<float>& part, unsigned* err) {
    if (gr.n > 63) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "weight gradient: grid above 63^3");
    if (cin == 16 && cout == 16) launch_conv_dw<16, 16>(ctx, gr, x, g, dw, db, part, err);
    else if (cin == 16 && cout == 32) launch_conv_dw<16, 32>(ctx, gr, x, g, dw, db, part, err);
    else if (cin == 32 && cout == 16) launch_conv_dw<32, 16>(ctx, gr, x, g, dw, db, part, err);
    else if (cin == 32 && cout == 32) launch_conv_dw<32, 32>(ctx, gr, x, g, dw, db, part, err);
    else throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "weight gradient: channel counts must be 16 or 32");
    ctx.check_launch("conv_dw_tc");
}

void planes_features(Context& ctx, const float* r, const float* c, const float* z, const float* scales, uint4* planes,
                     const VoxGrid& gr) {
    k_feat_planes<<<grid_for(ctx, (size_t)gr.n * gr.n * gr.n), 256, 0, ctx.stream>>>(r, c, z, scales, planes, gr);
    ctx.count_launch();
}

void planes_loss_grad(Context& ctx, const float* y32, const float* t, uint4* g, const VoxGrid& gr, float* loss) {
    k_loss_grad<<<grid_for(ctx, (size_t)gr.n * gr.n * gr.n), 256, 0, ctx.stream>>>(y32, t, g, gr, loss);
    ctx.count_launch();
}

void adam_step(Context& ctx, float* w, const float* g, float* m, float* v, size_t n, float lr, int t) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)t), c2 = 1.0f - std::pow(b2, (float)t);
    k_adam<<<grid_for(ctx, n), 256, 0, ctx.stream>>>(w, g, m, v, n, lr, b1, b2, 1e-8f, c1, c2);
    ctx.count_launch();
}

void pack_act(Context& ctx, const float* x, uint4* planes, const VoxGrid& g, int C) {
    const size_t work = (size_t)g.n * g.n * g.n * (C / 8);
    const unsigned grid = (unsigned)std::max<size_t>(1, std::min<size_t>((work + 255) / 256, (size_t)ctx.sm_count * 16));
    k_pack_act<<<grid, 256, 0, ctx.stream>>>(x, planes, g, C);
    ctx.count_launch();
}

void pack_weights(Context& ctx, const float* w, __nv_bfloat16* wg, int cin, int cout, bool flip) {
    const int total = 27 * cin * cout;
    k_pack_w<<<(total + 255) / 256, 256, 0, ctx.stream>>>(w, wg, cin, cout, flip ? 1 : 0);
    ctx.count_launch();
}

// One convolution from host buffers (diagnostic and test entry point).
void diag_conv3d(Context& ctx, int n, int cin, int cout, int flip, const float* x_h, const float* w_h,
                 const float* b_h, float* y_h) {
    if (n < 1) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "grid size must be positive");
    const int ci = flip ? cout : cin, co = flip ? cin : cout;  // channels of the convolution run
    const VoxGrid g = make_voxgrid(n);
    const size_t N = (size_t)n * n * n;
    DeviceArray<float> x(N * ci), w(27 * (size_t)cin * cout), b(co), y(N * co);
    DeviceArray<uint4> planes((size_t)(ci / 8) * g.rows);
    DeviceArray<__nv_bfloat16> wg(27 * (size_t)cin * cout);
    DeviceArray<unsigned> err(1);
    NUMA_CUDA(cudaMemsetAsync(planes.p, 0, planes.n * sizeof(uint4), ctx.stream));
    NUMA_CUDA(cudaMemsetAsync(err.p, 0, sizeof(unsigned), ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(x.p, x_h, N * ci * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(w.p, w_h, w.n * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    if (b_h) NUMA_CUDA(cudaMemcpyAsync(b.p, b_h, co * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    pack_act(ctx, x.p, planes.p, g, ci);
    pack_weights(ctx, w.p, wg.p, cin, cout, flip != 0);
    conv3d_tc(ctx, g, ci, co, planes.p, reinterpret_cast<const uint4*>(wg.p), b_h ? b.p : nullptr, nullptr, y.p, 0,
              err.p);
    unsigned herr = 0;
    NUMA_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(y_h, y.p, N * co * sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    if (herr) throw Status(NUMA_GPU_ERR_CUDA, "tensor-core convolution: an mbarrier wait gave up");
}

// One layer's weight and bias gradients from host buffers (diagnostic and test entry point):
// dw[tap][ci][co] = sum_v x[v + tap][ci] g[v][co], db[co] = sum_v g[v][co], x [n^3][cin], g [n^3][cout].
void diag_conv3d_wgrad(Context& ctx, int n, int cin, int cout, const float* x_h, const float* g_h, float* dw_h,
                       float* db_h) {
    if (n < 1) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "grid size must be positive");
    const VoxGrid g = make_voxgrid(n);
    const size_t N = (size_t)n * n * n;
    DeviceArray<float> x(N * cin), gr(N * cout), dw(27 * (size_t)cin * cout), db(cout), part;
    DeviceArray<uint4> xp((size_t)(cin / 8) * g.rows), gp((size_t)(cout / 8) * g.rows);
    DeviceArray<unsigned> err(1);
    NUMA_CUDA(cudaMemsetAsync(xp.p, 0, xp.n * sizeof(uint4), ctx.stream));
    NUMA_CUDA(cudaMemsetAsync(gp.p, 0, gp.n * sizeof(uint4), ctx.stream));
    NUMA_CUDA(cudaMemsetAsync(dw.p, 0, dw.n * sizeof(float), ctx.stream));
    NUMA_CUDA(cudaMemsetAsync(db.p, 0, db.n * sizeof(float), ctx.stream));
    NUMA_CUDA(cudaMemsetAsync(err.p, 0, sizeof(unsigned), ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(x.p, x_h, N * cin * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(gr.p, g_h, N * cout * sizeof(float), cudaMemcpyHostToDevice, ctx.stream));
    pack_act(ctx, x.p, xp.p, g, cin);
    pack_act(ctx, gr.p, gp.p, g, cout);
    conv_dw(ctx, g, cin, cout, xp.p, gp.p, dw.p, db.p, part, err.p);
    unsigned herr = 0;
    NUMA_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(dw_h, dw.p, dw.n * sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(db_h, db.p, db.n * sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    if (herr) throw Status(NUMA_GPU_ERR_CUDA, "tensor-core weight gradient: an mbarrier wait gave up");
}

}  // namespace numa::gpu
