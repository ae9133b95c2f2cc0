// gmres.cu — restarted right-preconditioned GMRES(m) and its recycled second solve
// (linalg/gmres.hpp) with the Krylov basis on the device.
//
// Per Arnoldi step j the device forms the Hessenberg column; the host reads that column (j+2
// doubles) once and runs the Givens rotations, the convergence test and the back-substitution
// in FP64 with the reference's exact arithmetic (gmres.hpp:155-196).
//
// Orthogonalisation:
//  * MGS (reference, gmres.hpp:141-144): one kernel per basis vector, each fusing the previous
//    axpy w -= h_{i-1} V_{i-1} (one FMA) with the next inner product <w, V_i>; the last one fuses
//    the final axpy with ||w||.  2(j+1)+1 FP64 operations per point, j+2 launches per step.
//  * CGS2: h = V^T w; w -= V h fused with h' = V^T w; w -= V h' fused with ||w||; H = h + h'.
//    Three passes over the basis, 4(j+1)+1 FP64 operations per point.
//  * CGS1: h = V^T w; w -= V h fused with ||w|| (2j + 5 vector passes).
// The fused classical Gram-Schmidt kernels keep one partial sum per basis vector in registers, for
// at most kCgsBlock vectors a pass; a longer basis is taken in blocks (updates of the earlier
// blocks chained through the output vector, dots of the earlier blocks after the last update),
// so a cycle runs to the restart length the caller asked for.
// On this GPU FP64 arithmetic, not bandwidth, bounds these kernels, so MGS is the cheaper of
// the two; CGS2 issues fewer launches and is the better-conditioned choice.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>

#include "numa_internal.hpp"

namespace numa::gpu {
namespace {

constexpr int kCgsBlock = 8;  // basis vectors per fused classical Gram-Schmidt pass

struct StoreAt {
    double* out;
    __device__ void operator()(const double (&t)[1]) const { *out = t[0]; }
};
struct StoreSqrtAt {
    double* out;
    __device__ void operator()(const double (&t)[1]) const { *out = __dsqrt_rn(t[0]); }
};

// w -= hprev * Vprev (when Vprev is given); accumulate <w, Vcur> (or ||w||^2 when Vcur is null).
template <bool HAS_PREV, bool NORM, class Fin>
__global__ void __launch_bounds__(kRedThreads) k_mgs(double* __restrict__ w, const double* __restrict__ Vprev,
                                                     const double* __restrict__ hprev,
                                                     const double* __restrict__ Vcur, size_t N, RedArgs red, Fin fin) {
    pdl_wait();
    pdl_trigger();
    __shared__ double sm[1][32];
    double s[1] = {0.0};
    const double a = HAS_PREV ? -(*hprev) : 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) {
        double wi = w[i];
        if (HAS_PREV) {
            wi = __fma_rn(a, Vprev[i], wi);
            w[i] = wi;
        }
        s[0] = NORM ? __fma_rn(wi, wi, s[0]) : __fma_rn(wi, Vcur[i], s[0]);
    }
    block_sum<1>(s, sm);
    grid_reduce_finish<1>(s, red, fin);
}

// CGS2 pieces.  V is (j+1) consecutive vectors of length ldv.
template <int R>
struct StoreVec {
    double* out;
    int cnt;
    __device__ void operator()(const double (&t)[R]) const {
        for (int r = 0; r < cnt; ++r) out[r] = t[r];
    }
};

__device__ __forceinline__ double widen(double v) { return v; }
__device__ __forceinline__ double widen(float v) { return f32_to_f64(v); }

// Fused classical Gram-Schmidt passes over CNT basis vectors (CNT a compile-time count, so the CNT
// partial sums stay in registers through the two-level reduction).  The vectors are v0 (r = 0) and
// V + r ldv (r >= 1), so a first vector can live outside the basis array.
// MODE 0: h[r] = <w, v_r>.
// MODE 1: wout = w - sum_r hin[r] sig2[r] v_r (sig2 = 1 when null), then h[r] = <wout, v_r>.
// MODE 2: the same wout, then h[0] = ||wout|| and, when sig2_out is given, *sig2_out = 1 / ||wout||^2
//         (0 for a zero vector).
// MODE 3: the same wout and no reduction (the earlier blocks of a basis longer than kCgsBlock).
// w and wout may be the same array (each element is read before it is written, by one thread).
template <int CNT, int MODE>
__global__ void __launch_bounds__(kRedThreads) k_cgs(const double* w, const double* __restrict__ v0,
                                                     const double* __restrict__ V, size_t ldv,
                                                     const double* __restrict__ hin, const double* __restrict__ sig2,
                                                     size_t N, RedArgs red, double* __restrict__ hout, double* wout,
                                                     double* __restrict__ sig2_out) {
    pdl_wait();
    pdl_trigger();
    constexpr int R = MODE == 2 ? 1 : CNT;
    __shared__ double sm[R][32];
    double hs[CNT];
#pragma unroll
    for (int r = 0; r < CNT; ++r) hs[r] = MODE != 0 ? hin[r] * (sig2 ? sig2[r] : 1.0) : 0.0;
    double s[R];
#pragma unroll
    for (int r = 0; r < R; ++r) s[r] = 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) {
        double wi = w[i];
        if (MODE != 0) {
#pragma unroll
            for (int r = 0; r < CNT; ++r) wi = __fma_rn(-hs[r], r == 0 ? v0[i] : V[(size_t)r * ldv + i], wi);
            wout[i] = wi;
        }
        if (MODE == 2) {
            s[0] = __fma_rn(wi, wi, s[0]);
        } else if (MODE != 3) {
#pragma unroll
            for (int r = 0; r < CNT; ++r) s[r] = __fma_rn(wi, r == 0 ? v0[i] : V[(size_t)r * ldv + i], s[r]);
        }
    }
    if constexpr (MODE != 3) {
        block_sum<R>(s, sm);
        grid_reduce_finish<R>(s, red, [hout, sig2_out] __device__(const double(&t)[R]) {
            if (MODE == 2) {
                const double nrm = __dsqrt_rn(t[0]);
                hout[0] = nrm;
                if (sig2_out) *sig2_out = t[0] > 0.0 ? 1.0 / t[0] : 0.0;
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) hout[r] = t[r];
            }
        });
    }
}

// Launches k_cgs<cnt, MODE> for 1 <= cnt <= kCgsBlock.
template <int MODE>
void launch_cgs(Context& ctx, int cnt, const double* w, const double* v0, const double* V, size_t N,
                const double* hin, const double* sig2, double* hout, double* wout, double* sig2_out) {
    const unsigned g = ctx.red_grid(N);
    switch (cnt) {
#define NUMA_CGS_CASE(K)                                                                                       \
    case K:                                                                                                    \
        launch_pdl(k_cgs<K, MODE>, g, kRedThreads, 0, ctx.stream, w, v0, V, N, hin, sig2, N, ctx.red, hout, wout,   \
                                                          sig2_out);                                         \
        break;
        NUMA_CGS_CASE(1)
        NUMA_CGS_CASE(2)
        NUMA_CGS_CASE(3)
        NUMA_CGS_CASE(4)
        NUMA_CGS_CASE(5)
        NUMA_CGS_CASE(6)
        NUMA_CGS_CASE(7)
        NUMA_CGS_CASE(8)
#undef NUMA_CGS_CASE
        default:
            throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "gmres: Gram-Schmidt block count outside 1..8");
    }
    ctx.count_launch();
}

// h[r] = <w, v_r> for r < cnt (v_0 = v0, v_r = V + r N): one fused pass per block of kCgsBlock.
void cgs_dots(Context& ctx, int cnt, const double* w, const double* v0, const double* V, size_t N, double* h,
              int upto = -1) {
    const int lim = upto < 0 ? cnt : upto;
    for (int b0 = 0; b0 < lim; b0 += kCgsBlock) {
        const int c = std::min(kCgsBlock, lim - b0);
        launch_cgs<0>(ctx, c, w, b0 == 0 ? v0 : V + (size_t)b0 * N, V + (size_t)b0 * N, N, nullptr, nullptr, h + b0,
                      nullptr, nullptr);
    }
}

// wout = w - sum_{r < cnt} hin[r] sig2[r] v_r (sig2 = 1 when null), then FIN = 2: hout[0] = ||wout||
// (and *sig2_out), or FIN = 1: hout[r] = <wout, v_r> for every r < cnt.  The earlier blocks update
// wout in place without a reduction; the last block fuses its update with the finish, and with
// FIN = 1 the dots of the earlier blocks follow on the finished wout.
template <int FIN>
void cgs_update(Context& ctx, int cnt, const double* w, const double* v0, const double* V, size_t N,
                const double* hin, const double* sig2, double* hout, double* wout, double* sig2_out) {
    const int nb = (cnt + kCgsBlock - 1) / kCgsBlock;
    const double* src = w;
    for (int bi = 0; bi < nb; ++bi) {
        const int b0 = bi * kCgsBlock, c = std::min(kCgsBlock, cnt - b0);
        const double* bv0 = b0 == 0 ? v0 : V + (size_t)b0 * N;
        const double* bV = V + (size_t)b0 * N;
        const double* bs = sig2 ? sig2 + b0 : nullptr;
        if (bi + 1 < nb) launch_cgs<3>(ctx, c, src, bv0, bV, N, hin + b0, bs, nullptr, wout, nullptr);
        else launch_cgs<FIN>(ctx, c, src, bv0, bV, N, hin + b0, bs, FIN == 1 ? hout + b0 : hout, wout, sig2_out);
        src = wout;
    }
    if (FIN == 1 && nb > 1) cgs_dots(ctx, cnt, wout, v0, V, N, hout, (nb - 1) * kCgsBlock);
}

// dst = src / d (gmres.hpp:128, :149) as src * RN(1/d): one FP64 instruction instead of a
// division (within 1.5 ulp of it; the basis vectors already differ from the reference's in the
// last bits through the order of the inner-product sums).
__global__ void k_div(const double* __restrict__ src, double d, double rd, double* __restrict__ dst, size_t N) {
    pdl_wait();
    pdl_trigger();
    (void)d;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) dst[i] = src[i] * rd;
}

// r = b - w (gmres.hpp:116)
__global__ void k_sub(const double* __restrict__ b, const double* __restrict__ w, double* __restrict__ r, size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) r[i] = b[i] - w[i];
}

// out = base + sum_i coef[i] * V_i, accumulated in i order per element as the reference's
// sequence of axpy calls does (gmres.hpp:198-199 with base = 0; :304-310 with base = b), each
// term fused into one FMA.
__global__ void k_combine(const double* __restrict__ base, const double* __restrict__ V, size_t ldv, int cnt,
                          const double* __restrict__ coef, double* __restrict__ out, size_t N) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ double cs[];
    for (int r = threadIdx.x; r < cnt; r += blockDim.x) cs[r] = coef[r];
    __syncthreads();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) {
        double t = base ? base[i] : 0.0;
        for (int r = 0; r < cnt; ++r) t = __fma_rn(cs[r], V[(size_t)r * ldv + i], t);
        out[i] = t;
    }
}

// x += sum_i coef[i] V_i in one pass (the flexible update; x is read and written in place); V in
// FP64, or in FP32 widened exactly (the same sums as from the widened vectors)
template <class VT>
__global__ void k_combine_add(const VT* __restrict__ V, size_t ldv, int cnt, const double* __restrict__ coef,
                              double* x, size_t N) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ double cs[];
    for (int r = threadIdx.x; r < cnt; r += blockDim.x) cs[r] = coef[r];
    __syncthreads();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) {
        double t = x[i];
        for (int r = 0; r < cnt; ++r) t = __fma_rn(cs[r], widen(V[(size_t)r * ldv + i]), t);
        x[i] = t;
    }
}

// ---- the FP32 basis (flexible GMRES with the FP32 hand-off and a loose linear tolerance).  The
// basis vectors u_j are FP32 and scaled to norms near 1; sigma_j = 1/||u_j|| (sig) and sigma_j^2
// (sig2) are device scalars.  Inner products and updates run in double-FP32 arithmetic on the
// FP32 pipe, so these passes are bound by HBM, not by the FP64 pipe.

// u0 = RN32(s * src): the first basis vector, normalised by s = 1/||src||
__global__ void k_to32_scaled(const double* __restrict__ src, double s, float* __restrict__ dst, size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride)
        dst[i] = f64_to_f32(__dmul_rn(src[i], s));
}

// Elements of each vector a thread loads ahead of the arithmetic in k_cgs_df.
template <int CNT>
constexpr int kCgsUnroll = CNT <= 2 ? 8 : (CNT <= 3 ? 4 : 2);

// MODE 0: h[r] = <w, u_r> for r < CNT.
// MODE 1: u = RN32(a (w - sum_r h[r] s2[r] u_r)) into uout (a = *ascale, or 1 when null), then
//         h[r] = <u, u_r> (the second pass of CGS2).
// MODE 2: the same u into uout, then hout[0] = ||u||, sig2[j+1] = 1/||u||^2, sig[j+1] = 1/||u||.
// MODE 3: the double-FP32 partial sum a w - sum_r a h[r] s2[r] u_r into part_out, no reduction (the
//         earlier blocks of a basis longer than kCgsBlock).
// With part_in given, MODES 1-3 start from that partial sum instead of a w.  In MODE 2 (CGS1, the
// second pass of CGS2 with a = sigma_j) the stored vectors keep norms near 1 in FP32 range.  Sums per
// thread in double-FP32, converted to FP64 for the block and grid reduction.  w and uout may be the
// same array, and so may part_in and part_out (each element is read before it is written, by one
// thread).
template <int CNT, int MODE>
__global__ void __launch_bounds__(kRedThreads) k_cgs_df(const float* w, const float2* part_in,
                                                        const float* __restrict__ u0, const float* __restrict__ U,
                                                        size_t ldu, const double* __restrict__ hin,
                                                        const double* __restrict__ s2c,
                                                        const double* __restrict__ ascale, double* sig2, double* sig,
                                                        int j, size_t N, RedArgs red, double* __restrict__ hout,
                                                        float* uout, float2* part_out) {
    pdl_wait();
    pdl_trigger();
    constexpr int R = MODE == 2 ? 1 : CNT;
    __shared__ double sm[R][32];
    DF cw{0.0f, 0.0f}, c[CNT];
    if (MODE != 0) {
        const double a = ascale ? *ascale : 1.0;
        cw = df_split(a);
#pragma unroll
        for (int r = 0; r < CNT; ++r) c[r] = df_split(-(a * hin[r] * s2c[r]));
    }
    DF acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = DF{0.0f, 0.0f};
    // One element: its w (or partial sum) and basis values already loaded.
    auto body = [&](size_t i, float wi, float2 pin, const float (&ur)[CNT]) {
        if (MODE == 0) {
#pragma unroll
            for (int r = 0; r < CNT; ++r) df_mac(acc[r], wi, ur[r]);
        } else {
            DF t{0.0f, 0.0f};
            if (part_in) t = DF{pin.x, pin.y};
            else df_mac(t, cw, wi);
#pragma unroll
            for (int r = 0; r < CNT; ++r) df_mac(t, c[r], ur[r]);
            if (MODE == 3) {
                part_out[i] = make_float2(t.hi, t.lo);
            } else {
                const float u = __fadd_rn(t.hi, t.lo);
                uout[i] = u;
                if (MODE == 2) {
                    df_mac(acc[0], u, u);
                } else {
#pragma unroll
                    for (int r = 0; r < CNT; ++r) df_mac(acc[r], u, ur[r]);
                }
            }
        }
    };
    auto load = [&](size_t i, float& wi, float2& pin, float (&ur)[CNT]) {
        if (MODE != 0 && part_in) pin = part_in[i];
        else wi = w[i];
#pragma unroll
        for (int r = 0; r < CNT; ++r) ur[r] = r == 0 ? u0[i] : U[(size_t)r * ldu + i];
    };
    // UF elements a thread an iteration, all their loads issued before any arithmetic: with one element a
    // thread the loads in flight were too few to cover DRAM latency (the passes ran at ~50 % of HBM).  Each
    // thread still visits its elements in the same order, so the sums are unchanged.
    constexpr int UF = kCgsUnroll<CNT>;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (; i + (UF - 1) * stride < N; i += UF * stride) {
        float wv[UF] = {}, uv[UF][CNT];
        float2 pv[UF] = {};
#pragma unroll
        for (int q = 0; q < UF; ++q) load(i + q * stride, wv[q], pv[q], uv[q]);
#pragma unroll
        for (int q = 0; q < UF; ++q) body(i + q * stride, wv[q], pv[q], uv[q]);
    }
    for (; i < N; i += stride) {
        float wi = 0.0f, ur[CNT];
        float2 pin = make_float2(0.0f, 0.0f);
        load(i, wi, pin, ur);
        body(i, wi, pin, ur);
    }
    if constexpr (MODE != 3) {
        double s[R];
#pragma unroll
        for (int r = 0; r < R; ++r) s[r] = df_to_f64(acc[r]);
        block_sum<R>(s, sm);
        grid_reduce_finish<R>(s, red, [hout, sig2, sig, j] __device__(const double(&t)[R]) {
            if (MODE == 2) {
                const double nrm = __dsqrt_rn(t[0]);
                hout[0] = nrm;
                sig2[j + 1] = t[0] > 0.0 ? 1.0 / t[0] : 0.0;
                sig[j + 1] = nrm > 0.0 ? 1.0 / nrm : 0.0;
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) hout[r] = t[r];
            }
        });
    }
}

// v 2^k for a power-of-two scale: the exponent field moved by integer addition where v and the result are
// normal numbers (exact either way), else the FP64 multiply (a call that is not inlined).
static __device__ __noinline__ double scale_pow2_rare(double v, double scale) { return __dmul_rn(v, scale); }
__device__ __forceinline__ double scale_pow2(double v, int k, double scale) {
    const int hi = __double2hiint(v);
    const int e = (hi >> 20) & 0x7FF;
    if (e == 0 || e + k < 1 || e + k > 2046) return scale_pow2_rare(v, scale);
    return __hiloint2double(hi + (k << 20), __double2loint(v));
}

// x += scale * sum_r coef[r] Z_r (ASSIGN: x = scale * sum_r coef[r] Z_r, x not read) with FP32 Z,
// |coef| <= 1 and scale = 2^k (the host normalises the coefficients by a power of two): the sum in
// double-FP32, widened by one FP64 addition and scaled exactly (ASSIGN), or added into x by one FMA.
// STEP (with ASSIGN): also xs = xb - x, the full Newton step from the value just stored.
template <int CNT, bool ASSIGN, bool STEP = false>
__global__ void k_combine_df(const float* __restrict__ Z, size_t ldz, const double* __restrict__ coef, double scale,
                             int kscale, double* x, size_t N, const double* __restrict__ xb = nullptr,
                             double* __restrict__ xs = nullptr) {
    pdl_wait();
    pdl_trigger();
    __shared__ DF cs[CNT];
    if (threadIdx.x < CNT) cs[threadIdx.x] = df_split(coef[threadIdx.x]);
    __syncthreads();
    DF c[CNT];
#pragma unroll
    for (int r = 0; r < CNT; ++r) c[r] = cs[r];
    // as in k_cgs_df: UF elements a thread an iteration, all loads first
    auto body = [&](size_t i, const float (&zr)[CNT], double xi, double xbi) {
        DF t{0.0f, 0.0f};
#pragma unroll
        for (int r = 0; r < CNT; ++r) df_mac(t, c[r], zr[r]);
        const double v = ASSIGN ? scale_pow2(df_to_f64(t), kscale, scale) : __fma_rn(scale, df_to_f64(t), xi);
        x[i] = v;
        if (STEP) xs[i] = xbi - v;
    };
    auto load = [&](size_t i, float (&zr)[CNT], double& xi, double& xbi) {
#pragma unroll
        for (int r = 0; r < CNT; ++r) zr[r] = Z[(size_t)r * ldz + i];
        if (!ASSIGN) xi = x[i];
        if (STEP) xbi = xb[i];
    };
    constexpr int UF = CNT <= 3 ? 4 : 2;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (; i + (UF - 1) * stride < N; i += UF * stride) {
        float zv[UF][CNT];
        double xv[UF] = {}, xbv[UF] = {};
#pragma unroll
        for (int q = 0; q < UF; ++q) load(i + q * stride, zv[q], xv[q], xbv[q]);
#pragma unroll
        for (int q = 0; q < UF; ++q) body(i + q * stride, zv[q], xv[q], xbv[q]);
    }
    for (; i < N; i += stride) {
        float zr[CNT];
        double xi = 0.0, xbi = 0.0;
        load(i, zr, xi, xbi);
        body(i, zr, xi, xbi);
    }
}

template <bool ASSIGN, bool STEP>
void launch_combine_df_block(Context& ctx, unsigned grid, int cnt, const float* Z, size_t N, const double* coef,
                             double scale, double* x, const double* xb, double* xs) {
    int kscale = 0;
    const double mant = std::frexp(scale, &kscale);  // scale = 2^(kscale - 1) when mant = 1/2
    if (mant != 0.5) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "gmres: the combine scale must be a power of two");
    kscale -= 1;
    switch (cnt) {
#define NUMA_COMBINE_DF_CASE(K)                                                                               \
    case K:                                                                                                   \
        launch_pdl(k_combine_df<K, ASSIGN, STEP>, grid, 256, 0, ctx.stream, Z, N, coef, scale, kscale, x, N, xb, \
                   xs);                                                                                       \
        break;
        NUMA_COMBINE_DF_CASE(1)
        NUMA_COMBINE_DF_CASE(2)
        NUMA_COMBINE_DF_CASE(3)
        NUMA_COMBINE_DF_CASE(4)
        NUMA_COMBINE_DF_CASE(5)
        NUMA_COMBINE_DF_CASE(6)
        NUMA_COMBINE_DF_CASE(7)
        NUMA_COMBINE_DF_CASE(8)
#undef NUMA_COMBINE_DF_CASE
        default:
            throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "gmres: combine block count outside 1..8");
    }
    ctx.count_launch();
}

// x (+)= scale sum_{r<cnt} coef_r Z_r in blocks of kCgsBlock vectors: the first block assigns (ASSIGN)
// or adds, later blocks add, and the last also writes the full step (STEP).
template <bool ASSIGN, bool STEP = false>
void launch_combine_df(Context& ctx, unsigned grid, int cnt, const float* Z, size_t N, const double* coef, double scale,
                       double* x, const double* xb = nullptr, double* xs = nullptr) {
    for (int b0 = 0; b0 < cnt; b0 += kCgsBlock) {
        const int c = std::min(kCgsBlock, cnt - b0);
        const bool first = b0 == 0, last = b0 + c >= cnt;
        const float* Zb = Z + (size_t)b0 * N;
        const double* cb = coef + b0;
        if (first && last) launch_combine_df_block<ASSIGN, STEP>(ctx, grid, c, Zb, N, cb, scale, x, xb, xs);
        else if (first) launch_combine_df_block<ASSIGN, false>(ctx, grid, c, Zb, N, cb, scale, x, xb, xs);
        else if (last) launch_combine_df_block<false, STEP>(ctx, grid, c, Zb, N, cb, scale, x, xb, xs);
        else launch_combine_df_block<false, false>(ctx, grid, c, Zb, N, cb, scale, x, xb, xs);
    }
}

// One wave of k_cgs_df<CNT, MODE>: the reduction grid, capped at the blocks that fit on the device at
// once (the longer unrolls hold more registers, and a second partial wave would double the pass).
template <int CNT, int MODE>
unsigned cgs_grid(Context& ctx, size_t N) {
    static std::atomic<int> per_sm{0};  // resident blocks an SM, found once
    int b = per_sm.load();
    if (b == 0) {
        NUMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_cgs_df<CNT, MODE>, kRedThreads, 0));
        b = b > 0 ? b : 1;
        per_sm.store(b);
    }
    return std::min(ctx.red_grid(N), (unsigned)(b * ctx.sm_count));
}

// Launches k_cgs_df<cnt, MODE> for 1 <= cnt <= kCgsBlock.
template <int MODE>
void launch_cgs_df(Context& ctx, int cnt, const float* w, const float2* part_in, const float* u0, const float* U,
                   size_t N, const double* hin, const double* s2c, const double* ascale, double* sig2, double* sig,
                   int j, double* hout, float* uout, float2* part_out) {
    switch (cnt) {
#define NUMA_CGS_DF_CASE(K)                                                                                  \
    case K:                                                                                                  \
        launch_pdl(k_cgs_df<K, MODE>, cgs_grid<K, MODE>(ctx, N), kRedThreads, 0, ctx.stream, w, part_in, \
                   u0, U, N, hin, s2c, ascale, sig2, sig, j, N, ctx.red, hout, uout, part_out);             \
        break;
        NUMA_CGS_DF_CASE(1)
        NUMA_CGS_DF_CASE(2)
        NUMA_CGS_DF_CASE(3)
        NUMA_CGS_DF_CASE(4)
        NUMA_CGS_DF_CASE(5)
        NUMA_CGS_DF_CASE(6)
        NUMA_CGS_DF_CASE(7)
        NUMA_CGS_DF_CASE(8)
#undef NUMA_CGS_DF_CASE
        default:
            throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "gmres: Gram-Schmidt block count outside 1..8");
    }
    ctx.count_launch();
}

// The FP32-basis forms of cgs_dots / cgs_update (u_0 = u0, u_r = U + r N).  cgs_update_df forms
// u = RN32(a (w - sum_r hin[r] s2[r] u_r)) into uout with FIN = 2 (norm and the sigma slots of j + 1)
// or FIN = 1 (h[r] = <u, u_r>); a basis longer than kCgsBlock chains its earlier blocks through the
// double-FP32 partial sums in part (2 floats a point).
void cgs_dots_df(Context& ctx, int cnt, const float* w, const float* u0, const float* U, size_t N, double* h,
                 int upto = -1) {
    const int lim = upto < 0 ? cnt : upto;
    for (int b0 = 0; b0 < lim; b0 += kCgsBlock) {
        const int c = std::min(kCgsBlock, lim - b0);
        launch_cgs_df<0>(ctx, c, w, nullptr, b0 == 0 ? u0 : U + (size_t)b0 * N, U + (size_t)b0 * N, N, nullptr,
                         nullptr, nullptr, nullptr, nullptr, 0, h + b0, nullptr, nullptr);
    }
}

template <int FIN>
void cgs_update_df(Context& ctx, int cnt, const float* w, const float* u0, const float* U, size_t N,
                   const double* hin, const double* s2, const double* ascale, double* sig2, double* sig, int j,
                   double* hout, float* uout, float2* part) {
    const int nb = (cnt + kCgsBlock - 1) / kCgsBlock;
    for (int bi = 0; bi < nb; ++bi) {
        const int b0 = bi * kCgsBlock, c = std::min(kCgsBlock, cnt - b0);
        const float* bu0 = b0 == 0 ? u0 : U + (size_t)b0 * N;
        const float* bU = U + (size_t)b0 * N;
        const float2* pin = bi == 0 ? nullptr : part;
        if (bi + 1 < nb)
            launch_cgs_df<3>(ctx, c, w, pin, bu0, bU, N, hin + b0, s2 + b0, ascale, sig2, sig, j, nullptr, nullptr,
                             part);
        else
            launch_cgs_df<FIN>(ctx, c, w, pin, bu0, bU, N, hin + b0, s2 + b0, ascale, sig2, sig, j,
                               FIN == 1 ? hout + b0 : hout, uout, nullptr);
    }
    if (FIN == 1 && nb > 1) cgs_dots_df(ctx, cnt, uout, u0, U, N, hout, (nb - 1) * kCgsBlock);
}

// *out = v (one device scalar from a host value, stream-ordered)
__global__ void k_set_scalar(double* __restrict__ out, double v) {
    pdl_wait();
    pdl_trigger();
    *out = v;
}

// Smallest linear tolerance for which FGMRES keeps its basis in FP32 (the FP32 hand-off only), with
// FP32-arithmetic products and with products of FP64 accuracy rounded to FP32 (GmresOptions::precise_tight).
constexpr double kV32MinRtol = 1e-5;
constexpr double kV32MinRtolPrecise = 1e-6;

unsigned ew_grid(const Context& ctx, size_t N) {
    size_t want = (N + 255) / 256;
    size_t cap = static_cast<size_t>(ctx.sm_count) * 16;
    if (want > cap) want = cap;
    return static_cast<unsigned>(want < 1 ? 1 : want);
}

}  // namespace

Gmres::Gmres(Context& ctx, size_t N) : ctx_(ctx), N_(N) {}

void Gmres::precond_apply(Precond* M, const double* r, double* z) {
    if (M) M->apply(r, z);
    else dev_copy(ctx_, r, z, N_);
}

// Leaves H[0..j][j] in hcol[0..j] and ||w|| in hcol[j+1]; w is orthogonalised in place.
void Gmres::arnoldi_mgs(size_t j, double* w) {
    double* hcol = ctx_.scalar(kSlotGmresH);
    const size_t N = N_;
    const unsigned g = ctx_.red_grid(N);
    const double* V = V_.p;
    launch_pdl(k_mgs<false, false, StoreAt>, g, kRedThreads, 0, ctx_.stream, w, nullptr, nullptr, V, N, ctx_.red, StoreAt{hcol});
    ctx_.count_launch();
    for (size_t i = 1; i <= j; ++i) {
        launch_pdl(k_mgs<true, false, StoreAt>, g, kRedThreads, 0, ctx_.stream, w, V + (i - 1) * N, hcol + (i - 1), V + i * N, N,
                                                              ctx_.red, StoreAt{hcol + i});
        ctx_.count_launch();
    }
    launch_pdl(k_mgs<true, true, StoreSqrtAt>, g, kRedThreads, 0, ctx_.stream, w, V + j * N, hcol + j, nullptr, N, ctx_.red,
                                                         StoreSqrtAt{hcol + j + 1});
    ctx_.count_launch();
    ctx_.check_launch("arnoldi mgs");
}

void Gmres::arnoldi_cgs2(size_t j, double* w) {
    double* hcol = ctx_.scalar(kSlotGmresH);
    double* h2 = ctx_.scalar(kSlotGmresH2);
    const size_t N = N_;
    const int cnt = (int)(j + 1);
    cgs_dots(ctx_, cnt, w, V_.p, V_.p, N, hcol);
    cgs_update<1>(ctx_, cnt, w, V_.p, V_.p, N, hcol, nullptr, h2, w, nullptr);
    cgs_update<2>(ctx_, cnt, w, V_.p, V_.p, N, h2, nullptr, hcol + j + 1, w, nullptr);
    ctx_.check_launch("arnoldi cgs2");
    // H = h + h' is formed on the host after the column is read (see solve).
}

// Classical Gram-Schmidt, one pass: h = V^T w in one multi-dot, then w -= V h and ||w|| in one
// update (2j + 5 vector passes against 4j + 5 for the fused MGS chain).  For the few Arnoldi steps a
// well-preconditioned solve takes, the loss of orthogonality is at rounding level.
void Gmres::arnoldi_cgs1(size_t j, double* w) {
    double* hcol = ctx_.scalar(kSlotGmresH);
    const size_t N = N_;
    const int cnt = (int)(j + 1);
    cgs_dots(ctx_, cnt, w, V_.p, V_.p, N, hcol);
    cgs_update<2>(ctx_, cnt, w, V_.p, V_.p, N, hcol, nullptr, hcol + j + 1, w, nullptr);
    ctx_.check_launch("arnoldi cgs1");
}

// Flexible GMRES with classical Gram-Schmidt (one pass, CGS1, or two, CGS2) and lazily normalised
// basis vectors: the basis keeps v~_j = w~ as the update pass writes it, with sigma_j = 1/||v~_j||
// (sigma_j^2 on the device, sigma_j on the host), so no pass divides a vector.  The preconditioned
// vectors are z_j := sigma_j M(v~_j) (FGMRES admits any z_j), A z_j = sigma_j A M(v~_j), and the
// Hessenberg entries and the final coefficients carry the sigmas: h_ij = sigma_j sigma_i
// <A M(v~_j), v~_i> (CGS2: plus the second pass' coefficients), h_{j+1,j} = sigma_j ||w~||,
// x += sum_j (y_j sigma_j) M(v~_j).  The first basis vector is the right-hand side (or residual)
// itself, read in place.  Cycles run to the restart length (the Gram-Schmidt passes take a long
// basis in blocks).
GmresResult Gmres::solve_lazy(LinearOp& A, Precond* M, const double* b, double* x, const GmresOptions& o,
                              const double* r_init) {
    const size_t N = N_;
    const size_t m = o.restart;
    if (m > kMaxRestart) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "GMRES restart larger than 250 is not supported");
    const bool two_pass = o.orth == NUMA_GPU_ORTH_CGS2;
    GmresResult res;
    double* sl = ctx_.scalar(kSlotGmresH);
    double* sig2 = ctx_.scalar(kSlotGmresSig2);
    double bnorm = o.bnorm;
    if (bnorm < 0.0) {
        dev_norm2(ctx_, b, N, sl);
        bnorm = ctx_.fetch1(sl);
    }
    if (bnorm == 0.0) {
        dev_fill(ctx_, x, 0.0, N);
        res.converged = true;
        return res;
    }
    if (o.restart == 0) {
        res.rel_res = 1.0;
        res.breakdown = true;
        return res;
    }
    if (o.max_iters == 0) {
        res.rel_res = 1.0;
        return res;
    }
    // a zero first guess is written by the first solution update itself (x = Z y, x not read); any
    // earlier exit or use of x fills it first
    bool x_zero_pending = o.zero_guess;
    auto settle_x = [&] {
        if (x_zero_pending) dev_fill(ctx_, x, 0.0, N);
        x_zero_pending = false;
    };
    // FP32 preconditioner output into an FP32 product: the preconditioned vectors are kept in FP32
    // (exactly the values the FP64 path would widen), halving their writes and reads
    const bool z32 = M && M->has_apply32() && A.has_apply32();
    // ... and, with a linear tolerance far above FP32 rounding (an inexact-Newton forcing term) and an
    // operator whose FP32 product can be stored as it is, the whole Arnoldi process runs on FP32
    // vectors: the basis u_0 = RN32(r / ||r||), u_1, ... and w = A z_j.  Rounding a stored vector
    // perturbs the Arnoldi relation A Z = V H by 6e-8 relative, which bounds the attainable linear
    // residual near that; inner products, updates and the solution update are computed in
    // double-FP32 and reduced in FP64, and the Hessenberg matrix and least squares stay FP64.
    // With products of FP64 accuracy (precise_tight): FP32 arithmetic in the Laplacian of a smooth vector loses
    // digits to cancellation and bounds the attainable true residual well above a tight tolerance, while a
    // product computed accurately and rounded once to FP32 perturbs it by 6e-8 relative, like the stored basis.
    // So between 1e-6 and 1e-5 the basis stays FP32 with those products; below 1e-6 it is FP64 and the products
    // are kept in FP64.
    const bool can_precise = z32 && o.precise_tight && A.has_apply32x();
    const bool v32 = z32 && M->has_apply32f() && A.has_apply32f() &&
                     o.rtol >= (can_precise ? kV32MinRtolPrecise : kV32MinRtol);
    const bool precise = can_precise && !v32;
    const bool precise_v32 = can_precise && v32 && o.rtol < kV32MinRtol;
    double* sigd = ctx_.scalar(kSlotGmresSig);
    if (v32) {
        V32_.resize((m + 1) * N);
        W32_.resize(N);
        if (m + 1 > (size_t)kCgsBlock) P32_.resize(2 * N);  // double-FP32 partial sums of a long basis
    } else {
        V_.resize((m + 1) * N);
    }
    if (z32) Z32_.resize(m * N);
    else Z_.resize(m * N);
    w_.resize(N);
    r_.resize(N);
    std::vector<std::vector<double>> H(m + 1, std::vector<double>(m, 0.0));
    std::vector<double> cs(m), sn(m), g(m + 1), y(m), col(m + 2), col2(m + 1), sig(m + 1);
    double* ydev = ctx_.scalar(kSlotGmresY);
    double* h2 = ctx_.scalar(kSlotGmresH2);
    float2* part = v32 && m + 1 > (size_t)kCgsBlock ? reinterpret_cast<float2*>(P32_.p) : nullptr;
    bool given = r_init != nullptr;
    bool first = o.zero_guess;
    const unsigned eg = ew_grid(ctx_, N);
    while (res.iters < o.max_iters) {
        const double* v0;
        const float* v0_32 = nullptr;  // RN32(v0) from the caller, used as it is
        double beta;
        if (given) {
            v0 = r_init;
            given = false;
            first = false;
            dev_norm2(ctx_, v0, N, sl);
            beta = ctx_.fetch1(sl);
        } else if (first) {
            v0 = b;
            first = false;
            beta = bnorm;
            // elements of order beta / sqrt(N): far from FP32's range limits for the double-FP32 products
            const double typ = beta / std::sqrt((double)N);
            if (o.b32 && typ > 1e-15 && typ < 1e15) v0_32 = o.b32;
        } else {
            settle_x();
            A.apply(x, w_.p);
            ++res.matvecs;
            launch_pdl(k_sub, eg, 256, 0, ctx_.stream, b, w_.p, r_.p, N);
            ctx_.count_launch();
            v0 = r_.p;
            dev_norm2(ctx_, v0, N, sl);
            beta = ctx_.fetch1(sl);
        }
        res.rel_res = beta / bnorm;
        if (res.rel_res <= o.rtol) {
            res.converged = true;
            settle_x();
            break;
        }
        if (v32 && v0_32) {
            // u_0 = RN32(b) as the caller stored it, sigma_0 = 1/||b||: no conversion pass
            launch_pdl(k_set_scalar, 1, 1, 0, ctx_.stream, sig2, 1.0 / (beta * beta));
            launch_pdl(k_set_scalar, 1, 1, 0, ctx_.stream, sigd, 1.0 / beta);
            ctx_.count_launch(2);
            sig[0] = 1.0 / beta;
        } else if (v32) {
            launch_pdl(k_to32_scaled, eg, 256, 0, ctx_.stream, v0, 1.0 / beta, V32_.p, N);
            launch_pdl(k_set_scalar, 1, 1, 0, ctx_.stream, sig2, 1.0);
            launch_pdl(k_set_scalar, 1, 1, 0, ctx_.stream, sigd, 1.0);
            ctx_.count_launch(3);
            sig[0] = 1.0;
        } else {
            launch_pdl(k_set_scalar, 1, 1, 0, ctx_.stream, sig2, 1.0 / (beta * beta));
            ctx_.count_launch();
            sig[0] = 1.0 / beta;
        }
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        const float* u0 = v0_32 ? v0_32 : V32_.p;  // the FP32 basis' first vector
        size_t k = 0;
        while (k < m && res.iters < o.max_iters) {
            const size_t j = k;
            const double* vj = v32 ? nullptr : (j == 0 ? v0 : V_.p + j * N);
            if (v32) {
                float* zj = Z32_.p + j * N;
                M->apply32f(j == 0 ? u0 : V32_.p + j * N, zj);
                ++res.precs;
                if (precise_v32) A.apply32xf(zj, W32_.p);
                else A.apply32f(zj, W32_.p);
            } else if (z32) {
                float* zj = Z32_.p + j * N;
                M->apply32(vj, zj);
                ++res.precs;
                if (precise) A.apply32x(zj, w_.p);
                else A.apply32(zj, w_.p);
            } else {
                double* zj = Z_.p + j * N;
                precond_apply(M, vj, zj);
                ++res.precs;
                A.apply(zj, w_.p);
            }
            ++res.matvecs;
            const int cnt = (int)(j + 1);
            float* unext = v32 ? V32_.p + (j + 1) * N : nullptr;
            if (v32 && !two_pass) {
                cgs_dots_df(ctx_, cnt, W32_.p, u0, V32_.p, N, sl);
                cgs_update_df<2>(ctx_, cnt, W32_.p, u0, V32_.p, N, sl, sig2, sigd + j, sig2, sigd, (int)j, sl + j + 1,
                                 unext, part);
            } else if (v32) {
                // w' = RN32(sigma_j (w - sum c_r sigma_r^2 u_r)) into the next slot with c'_r = <w', u_r>, then
                // u_{j+1} = RN32(w' - sum c'_r sigma_r^2 u_r) in place
                cgs_dots_df(ctx_, cnt, W32_.p, u0, V32_.p, N, sl);
                cgs_update_df<1>(ctx_, cnt, W32_.p, u0, V32_.p, N, sl, sig2, sigd + j, sig2, sigd, (int)j, h2, unext,
                                 part);
                cgs_update_df<2>(ctx_, cnt, unext, u0, V32_.p, N, h2, sig2, nullptr, sig2, sigd, (int)j, sl + j + 1,
                                 unext, part);
            } else if (!two_pass) {
                cgs_dots(ctx_, cnt, w_.p, v0, V_.p, N, sl);
                cgs_update<2>(ctx_, cnt, w_.p, v0, V_.p, N, sl, sig2, sl + j + 1, V_.p + (j + 1) * N, sig2 + j + 1);
            } else {
                cgs_dots(ctx_, cnt, w_.p, v0, V_.p, N, sl);
                cgs_update<1>(ctx_, cnt, w_.p, v0, V_.p, N, sl, sig2, h2, w_.p, nullptr);
                cgs_update<2>(ctx_, cnt, w_.p, v0, V_.p, N, h2, sig2, sl + j + 1, V_.p + (j + 1) * N, sig2 + j + 1);
            }
            ctx_.check_launch("arnoldi (lazy cgs)");
            ctx_.fetch(sl, (int)(j + 2), col.data());
            if (two_pass) ctx_.fetch(h2, (int)(j + 1), col2.data());
            for (size_t i = 0; i <= j; ++i) H[i][j] = sig[j] * sig[i] * col[i];
            // the second pass' coefficients: on sigma_j w~ (FP32 basis) or on w~ itself
            if (two_pass)
                for (size_t i = 0; i <= j; ++i) H[i][j] += v32 ? sig[i] * col2[i] : sig[j] * sig[i] * col2[i];
            H[j + 1][j] = v32 ? col[j + 1] : sig[j] * col[j + 1];  // the FP32 u_{j+1} carries sigma_j
            sig[j + 1] = col[j + 1] > 0.0 ? 1.0 / col[j + 1] : 0.0;
            for (size_t i = 0; i < j; ++i) {
                const double t = cs[i] * H[i][j] + sn[i] * H[i + 1][j];
                H[i + 1][j] = -sn[i] * H[i][j] + cs[i] * H[i + 1][j];
                H[i][j] = t;
            }
            const double den = std::hypot(H[j][j], H[j + 1][j]);
            if (!(den > 0.0) || !std::isfinite(den)) {
                res.breakdown = true;
                settle_x();
                return res;
            }
            cs[j] = H[j][j] / den;
            sn[j] = H[j + 1][j] / den;
            H[j][j] = den;
            H[j + 1][j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            ++k;
            ++res.iters;
            res.rel_res = std::abs(g[j + 1]) / bnorm;
            if (M) M->progress(res.iters, res.rel_res);
            if (res.rel_res <= o.rtol) break;
        }
        for (size_t ii = k; ii-- > 0;) {
            const double piv = H[ii][ii];
            if (!(std::abs(piv) > 0.0) || !std::isfinite(piv)) {
                res.breakdown = true;
                settle_x();
                return res;
            }
            double t = g[ii];
            for (size_t jj = ii + 1; jj < k; ++jj) t -= H[ii][jj] * y[jj];
            y[ii] = t / piv;
        }
        double* yh = pin_.get(m);
        for (size_t jj = 0; jj < k; ++jj) yh[jj] = y[jj] * sig[jj];
        double scale = 1.0;  // a power of two at or above max |yh|: the division is exact
        if (v32) {
            double amax = 0.0;
            for (size_t jj = 0; jj < k; ++jj) amax = std::max(amax, std::abs(yh[jj]));
            if (amax > 0.0 && std::isfinite(amax)) {
                int e = 0;
                std::frexp(amax, &e);  // amax < 2^e
                scale = std::ldexp(1.0, e);
                for (size_t jj = 0; jj < k; ++jj) yh[jj] /= scale;
            }
        }
        NUMA_CUDA(cudaMemcpyAsync(ydev, yh, k * sizeof(double), cudaMemcpyHostToDevice, ctx_.stream));
        if (v32) {
            if (x_zero_pending && o.x_step) {
                launch_combine_df<true, true>(ctx_, eg, (int)k, Z32_.p, N, ydev, scale, x, o.x_base, o.x_step);
                res.stepped = true;
            } else {
                if (x_zero_pending) launch_combine_df<true>(ctx_, eg, (int)k, Z32_.p, N, ydev, scale, x);
                else launch_combine_df<false>(ctx_, eg, (int)k, Z32_.p, N, ydev, scale, x);
                res.stepped = false;  // a later update: the step written before no longer matches x
            }
            x_zero_pending = false;
        } else {
            settle_x();
            if (z32) launch_pdl(k_combine_add<float>, eg, 256, k * sizeof(double), ctx_.stream, Z32_.p, N, (int)k, ydev, x, N);
            else launch_pdl(k_combine_add<double>, eg, 256, k * sizeof(double), ctx_.stream, Z_.p, N, (int)k, ydev, x, N);
            ctx_.count_launch();
        }
        ctx_.check_launch("gmres update (lazy)");
        if (res.rel_res <= o.rtol) {
            res.converged = true;
            break;
        }
    }
    settle_x();
    return res;
}

GmresResult Gmres::solve(LinearOp& A, Precond* M, const double* b, double* x, const GmresOptions& o,
                         KrylovSpace* save, const double* r_init) {
    if (o.flexible && (o.orth == NUMA_GPU_ORTH_CGS1 || o.orth == NUMA_GPU_ORTH_CGS2) && !save)
        return solve_lazy(A, M, b, x, o, r_init);
    const size_t N = N_;
    const size_t m = o.restart;
    GmresResult res;
    if (save) save->clear();

    double* sl = ctx_.scalar(kSlotGmresH);
    dev_norm2(ctx_, b, N, sl);
    const double bnorm = ctx_.fetch1(sl);
    if (bnorm == 0.0) {
        dev_fill(ctx_, x, 0.0, N);
        res.converged = true;
        return res;
    }
    if (m == 0) {
        res.rel_res = 1.0;
        res.breakdown = true;
        return res;
    }
    if (o.max_iters == 0) {
        res.rel_res = 1.0;
        return res;
    }
    if (m > kMaxRestart) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "GMRES restart larger than 250 is not supported");
    if (o.zero_guess) dev_fill(ctx_, x, 0.0, N);

    const bool cgs2 = o.orth == NUMA_GPU_ORTH_CGS2;
    const bool cgs1 = o.orth == NUMA_GPU_ORTH_CGS1;
    V_.resize((m + 1) * N);
    if (o.flexible) Z_.resize(m * N);
    w_.resize(N);
    r_.resize(N);
    comb_.resize(N);
    z_.resize(N);

    std::vector<std::vector<double>> H(m + 1, std::vector<double>(m, 0.0));
    std::vector<std::vector<double>> Hraw(m + 1, std::vector<double>(m, 0.0));
    std::vector<double> cs(m), sn(m), g(m + 1), y(m), col(m + 2), col2(m + 2);
    double* ydev = ctx_.scalar(kSlotGmresY);

    bool given = r_init != nullptr;
    bool first = o.zero_guess;
    size_t k_last = 0;
    const unsigned eg = ew_grid(ctx_, N);

    while (res.iters < o.max_iters) {
        const double* rv;
        if (given) {
            rv = r_init;
            given = false;
            first = false;
        } else if (first) {
            rv = b;
            first = false;
        } else {
            A.apply(x, w_.p);
            ++res.matvecs;
            launch_pdl(k_sub, eg, 256, 0, ctx_.stream, b, w_.p, r_.p, N);
            ctx_.count_launch();
            rv = r_.p;
        }
        dev_norm2(ctx_, rv, N, sl);
        const double beta = ctx_.fetch1(sl);
        res.rel_res = beta / bnorm;
        if (res.rel_res <= o.rtol) {
            res.converged = true;
            k_last = 0;
            break;
        }
        for (auto& row : Hraw) std::fill(row.begin(), row.end(), 0.0);
        launch_pdl(k_div, eg, 256, 0, ctx_.stream, rv, beta, 1.0 / beta, V_.p, N);
        ctx_.count_launch();
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;

        size_t k = 0;
        k_last = 0;
        while (k < m && res.iters < o.max_iters) {
            const size_t j = k;
            double* zj = o.flexible ? Z_.p + j * N : z_.p;
            precond_apply(M, V_.p + j * N, zj);
            ++res.precs;
            A.apply(zj, w_.p);
            ++res.matvecs;
            if (cgs2) {
                arnoldi_cgs2(j, w_.p);
                ctx_.fetch(sl, (int)(j + 2), col.data());
                ctx_.fetch(ctx_.scalar(kSlotGmresH2), (int)(j + 1), col2.data());
                for (size_t i = 0; i <= j; ++i) col[i] += col2[i];
            } else if (cgs1) {
                arnoldi_cgs1(j, w_.p);
                ctx_.fetch(sl, (int)(j + 2), col.data());
            } else {
                arnoldi_mgs(j, w_.p);
                ctx_.fetch(sl, (int)(j + 2), col.data());
            }
            for (size_t i = 0; i <= j + 1; ++i) H[i][j] = col[i];
            double* vnext = V_.p + (j + 1) * N;
            if (H[j + 1][j] > 0.0) {
                launch_pdl(k_div, eg, 256, 0, ctx_.stream, w_.p, H[j + 1][j], 1.0 / H[j + 1][j], vnext, N);
                ctx_.count_launch();
            } else {
                dev_fill(ctx_, vnext, 0.0, N);
            }
            for (size_t i = 0; i <= j + 1; ++i) Hraw[i][j] = H[i][j];
            for (size_t i = 0; i < j; ++i) {
                const double t = cs[i] * H[i][j] + sn[i] * H[i + 1][j];
                H[i + 1][j] = -sn[i] * H[i][j] + cs[i] * H[i + 1][j];
                H[i][j] = t;
            }
            const double den = std::hypot(H[j][j], H[j + 1][j]);
            if (!(den > 0.0) || !std::isfinite(den)) {
                res.breakdown = true;
                return res;
            }
            cs[j] = H[j][j] / den;
            sn[j] = H[j + 1][j] / den;
            H[j][j] = den;
            H[j + 1][j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            ++k;
            ++res.iters;
            k_last = k;
            res.rel_res = std::abs(g[j + 1]) / bnorm;
            if (M) M->progress(res.iters, res.rel_res);
            if (res.rel_res <= o.rtol) break;
        }
        for (size_t ii = k; ii-- > 0;) {
            const double piv = H[ii][ii];
            if (!(std::abs(piv) > 0.0) || !std::isfinite(piv)) {
                res.breakdown = true;
                return res;
            }
            double s = g[ii];
            for (size_t jj = ii + 1; jj < k; ++jj) s -= H[ii][jj] * y[jj];
            y[ii] = s / piv;
        }
        double* yh = pin_.get(m);
        std::memcpy(yh, y.data(), k * sizeof(double));
        NUMA_CUDA(cudaMemcpyAsync(ydev, yh, k * sizeof(double), cudaMemcpyHostToDevice, ctx_.stream));
        if (o.flexible) {
            launch_pdl(k_combine, eg, 256, k * sizeof(double), ctx_.stream, nullptr, Z_.p, N, (int)k, ydev, comb_.p, N);
            ctx_.count_launch();
            dev_axpy(ctx_, 1.0, comb_.p, x, N);
        } else {
            launch_pdl(k_combine, eg, 256, k * sizeof(double), ctx_.stream, nullptr, V_.p, N, (int)k, ydev, comb_.p, N);
            ctx_.count_launch();
            precond_apply(M, comb_.p, z_.p);
            ++res.precs;
            dev_axpy(ctx_, 1.0, z_.p, x, N);
        }
        // (the pinned y buffer is next written after a later fetch has synchronised the stream)
        ctx_.check_launch("gmres update");
        if (res.rel_res <= o.rtol) {
            res.converged = true;
            break;
        }
    }
    if (save && k_last > 0) {
        save->k = k_last;
        save->N = N;
        save->V.swap(V_);
        save->Hbar.assign(k_last + 1, std::vector<double>(k_last, 0.0));
        for (size_t i = 0; i <= k_last; ++i)
            for (size_t j = 0; j < k_last; ++j) save->Hbar[i][j] = Hraw[i][j];
    }
    return res;
}

GmresResult Gmres::solve_recycled(LinearOp& A, Precond* M, const double* b, double* x, const GmresOptions& o,
                                  const KrylovSpace& sp, KrylovSpace* save) {
    const size_t k = sp.k, N = N_;
    dev_fill(ctx_, x, 0.0, N);
    GmresOptions fresh = o;
    fresh.zero_guess = true;
    bool usable = k > 0 && sp.N == N && sp.Hbar.size() >= k + 1 && sp.V.n >= (k + 1) * N;
    if (usable)
        for (size_t i = 0; i <= k; ++i)
            if (sp.Hbar[i].size() < k) usable = false;
    if (!usable) return solve(A, M, b, x, fresh, save);
    if (k > kMaxRestart) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "recycled space too large");

    // rhs_i = <V_i, b> (gmres.hpp:252-255)
    double* sl = ctx_.scalar(kSlotGmresH);
    for (size_t i = 0; i <= k; ++i) dev_dot(ctx_, sp.V.p + i * N, b, N, sl + i);
    std::vector<double> rhs(k + 1);
    ctx_.fetch(sl, (int)(k + 1), rhs.data());

    auto R = sp.Hbar;
    std::vector<double> cs(k, 0.0), sn(k, 0.0);
    for (size_t j = 0; j < k; ++j) {
        for (size_t i = 0; i < j; ++i) {
            const double t = cs[i] * R[i][j] + sn[i] * R[i + 1][j];
            R[i + 1][j] = -sn[i] * R[i][j] + cs[i] * R[i + 1][j];
            R[i][j] = t;
        }
        const double den = std::hypot(R[j][j], R[j + 1][j]);
        if (!(den > 0.0) || !std::isfinite(den)) return solve(A, M, b, x, fresh, save);
        cs[j] = R[j][j] / den;
        sn[j] = R[j + 1][j] / den;
        R[j][j] = den;
        R[j + 1][j] = 0.0;
        const double t = cs[j] * rhs[j] + sn[j] * rhs[j + 1];
        rhs[j + 1] = -sn[j] * rhs[j] + cs[j] * rhs[j + 1];
        rhs[j] = t;
    }
    std::vector<double> y(k, 0.0);
    for (size_t ii = k; ii-- > 0;) {
        const double piv = R[ii][ii];
        if (!(std::abs(piv) > 0.0) || !std::isfinite(piv)) {
            dev_fill(ctx_, x, 0.0, N);
            return solve(A, M, b, x, fresh, save);
        }
        double s = rhs[ii];
        for (size_t jj = ii + 1; jj < k; ++jj) s -= R[ii][jj] * y[jj];
        y[ii] = s / piv;
    }
    // residual = b - sum_i (Hbar y)_i V_i, one axpy per i in i order (gmres.hpp:304-310)
    std::vector<double> coef(2 * k + 1);
    for (size_t i = 0; i <= k; ++i) {
        double c = 0.0;
        for (size_t j = 0; j < k; ++j) c += sp.Hbar[i][j] * y[j];
        coef[i] = -c;
    }
    for (size_t j = 0; j < k; ++j) coef[k + 1 + j] = y[j];
    double* ch = pin_.get(2 * k + 1);
    std::memcpy(ch, coef.data(), (2 * k + 1) * sizeof(double));
    double* cdev = ctx_.scalar(kSlotGmresCoef);
    NUMA_CUDA(cudaMemcpyAsync(cdev, ch, (2 * k + 1) * sizeof(double), cudaMemcpyHostToDevice, ctx_.stream));
    rrec_.resize(N);
    comb_.resize(N);
    const unsigned eg = ew_grid(ctx_, N);
    launch_pdl(k_combine, eg, 256, (k + 1) * sizeof(double), ctx_.stream, b, sp.V.p, N, (int)(k + 1), cdev, rrec_.p, N);
    // comb = sum_{j<k} y_j V_j; x = M comb (gmres.hpp:312-317)
    launch_pdl(k_combine, eg, 256, k * sizeof(double), ctx_.stream, nullptr, sp.V.p, N, (int)k, cdev + k + 1, comb_.p, N);
    ctx_.count_launch(2);
    NUMA_CUDA(cudaStreamSynchronize(ctx_.stream));
    precond_apply(M, comb_.p, x);
    GmresOptions cont = o;
    cont.zero_guess = false;
    GmresResult out = solve(A, M, b, x, cont, save, rrec_.p);
    ++out.precs;
    return out;
}

}  // namespace numa::gpu
