// common.cuh — shared device helpers and the host-side context of libnuma_gpu.
//
// Design notes for GB300 (sm_103a):
//  * FP64 arithmetic runs at ~1.2 TFLOP/s on this part (measured), 1/58 of FP32, so every FP64
//    kernel here is bound by its FP64 instruction count, not by HBM.  Kernels therefore avoid
//    redundant FP64 work (no halo recomputation, cached lambda*e^u, precomputed b*h^2, the
//    3-operation correctly-rounded division by 6 below) and trade memory traffic for FP64 ops.
//  * FP32 kernels (the mixed-precision V-cycle) are bound by HBM bandwidth.
//  * The library is built with -fmad=false: no multiply-add is contracted unless written as an
//    explicit fma, so element-wise results follow the reference's IEEE operation sequence.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <utility>
#include <stdexcept>
#include <string>

#include "../../include/numa_gpu.h"

namespace numa::gpu {

// ------------------------------------------------------------------------------------------
// Errors: internal code throws Status; the C ABI converts it to an int status code.
struct Status : std::runtime_error {
    int code;
    Status(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

[[noreturn]] void throw_cuda(cudaError_t e, const char* what, const char* file, int line);

#define NUMA_CUDA(expr)                                                              \
    do {                                                                             \
        cudaError_t numa_cuda_err_ = (expr);                                         \
        if (numa_cuda_err_ != cudaSuccess)                                           \
            ::numa::gpu::throw_cuda(numa_cuda_err_, #expr, __FILE__, __LINE__);      \
    } while (0)

// ------------------------------------------------------------------------------------------
// Reduction protocol.  A reducing kernel accumulates per-thread FP64 sums, reduces them within
// the block (warp shuffles, then shared memory), writes one partial per block and result, and
// takes a ticket; the last block to arrive sums the partials in block order and calls the
// kernel's finaliser.  The summation order depends only on the launch shape, so results are
// reproducible run to run.
constexpr int kMaxRedBlocks = 8192;   // partials per result
constexpr int kMaxRedResults = 64;    // results per reducing kernel (multi-dot width)
constexpr int kRedThreads = 256;

struct RedArgs {
    double* partials;   // kMaxRedBlocks * kMaxRedResults
    unsigned* ticket;   // one counter, reset to 0 by the last block
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of R values per thread; every thread of the block must call it.  Returns the
// block totals in warp 0 lane 0 (others hold unspecified values).
template <int R>
__device__ __forceinline__ void block_sum(double (&v)[R], double (*smem)[32]) {
    const int lane = threadIdx.x & 31;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int warp = tid >> 5;
    const int nwarps = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        double s = warp_sum(v[r]);
        if ((tid & 31) == 0) smem[r][warp] = s;
    }
    (void)lane;
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            double s = (tid < nwarps) ? smem[r][tid] : 0.0;
            v[r] = warp_sum(s);
        }
    }
    __syncthreads();
}

// Publishes this block's totals and, in the last block to finish, reduces all partials and
// calls fin(totals) on thread 0.  `v` must hold the block totals in thread 0 (block_sum output).
template <int R, class Fin>
__device__ __forceinline__ void grid_reduce_finish(const double (&v)[R], RedArgs red, Fin fin) {
    __shared__ bool am_last;
    __shared__ double tot_smem[R][32];
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
    const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    if (tid == 0) {
#pragma unroll
        for (int r = 0; r < R; ++r) red.partials[(size_t)r * kMaxRedBlocks + bid] = v[r];
        __threadfence();
        const unsigned t = atomicAdd(red.ticket, 1u);
        am_last = (t == nblocks - 1);
    }
    __syncthreads();
    if (!am_last) return;
    __threadfence();
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
    double acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        double s = 0.0;
        for (unsigned b = tid; b < nblocks; b += nthreads) s += __ldcg(red.partials + (size_t)r * kMaxRedBlocks + b);
        acc[r] = s;
    }
    block_sum<R>(acc, tot_smem);
    if (tid == 0) {
        fin(acc);
        *red.ticket = 0u;
    }
}

// ------------------------------------------------------------------------------------------
// Correctly rounded s / 6 in two FP64 operations (N. Brisebarre, J.-M. Muller, S. K. Raina,
// "Accelerating correctly rounded floating-point division when the divisor is known in advance",
// IEEE Trans. Computers 53(8), 2004): with 1/6 = zh + zl (zh = RN(1/6), zl = RN(1/6 - zh)),
// RN(s zh + RN(s zl)) by one multiply and one FMA.  Before the final rounding the value is within
// 2^-106 |s| of s/6, while s/6 is never closer than ~2^-58 |s/6| to a rounding midpoint (six times a
// 54-bit midpoint differs from every 53-bit s by an odd multiple of its last place), so the result
// is the IEEE quotient for every s with |s| >= 2^-960 (below, s zl underflows); checked against
// IEEE division on 2.1e9 random operands on the CPU and through the bit-exact V-cycle tests on the
// GPU.  (The three-operation Markstein form it replaces had the same kind of small-value limit.)
__device__ __forceinline__ double div6(double s) {
    return __fma_rn(s, 0x1.5555555555555p-3, __dmul_rn(s, 0x1.5555555555555p-57));
}
__device__ __forceinline__ float div6(float s) {
    const float r = 0.16666667f;
    const float q = __fmul_rn(s, r);
    const float e = __fmaf_rn(-q, 6.0f, s);
    return __fmaf_rn(e, r, q);
}

// a / d given rd = RN(1/d): the same correction for a runtime divisor.  Within one ulp of IEEE
// division and equal to it for all but rare (a, d) pairs.
__device__ __forceinline__ double div_by(double a, double d, double rd) {
    const double q = __dmul_rn(a, rd);
    const double e = __fma_rn(-q, d, a);
    return __fma_rn(e, rd, q);
}

// ------------------------------------------------------------------------------------------
// FP64 <-> FP32 conversions in integer arithmetic.  On this GPU the hardware conversion
// instructions issue on the (slow) FP64 pipe; these use only integer instructions and give the
// same results: round-to-nearest-even from the IEEE-754 bit fields, with the rare cases (float
// subnormals, NaN) handed to the hardware instruction.
// The hardware conversions for the rare operands (float subnormals, infinities, NaN) sit in calls
// that are not inlined, so the compiler branches around them instead of predicating them: a
// conversion involving FP64 issues on the FP64 pipe, which would otherwise be paid by every element.
static __device__ __noinline__ float f64_to_f32_rare(double d) { return __double2float_rn(d); }
static __device__ __noinline__ double f32_to_f64_rare(float f) { return (double)f; }

__device__ __forceinline__ float f64_to_f32(double d) {
    const unsigned hi = (unsigned)__double2hiint(d);
    const unsigned lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7FFu);
    const int ef = e - 896;  // re-biased exponent (1023 -> 127)
    if (ef >= 1 && ef < 255) {
        unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // top 23 fraction bits
        const unsigned rem = lo & 0x1FFFFFFFu;             // the 29 bits dropped
        unsigned bits = ((unsigned)ef << 23) | m;
        bits += (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;  // carries into the exponent
        if (bits >= 0x7F800000u) bits = 0x7F800000u;                                // overflow to infinity
        return __uint_as_float(sign | bits);
    }
    if (e == 0 || ef <= -25) return __uint_as_float(sign);  // zero, or too small for a float subnormal
    if (ef >= 255 && e != 0x7FF) return __uint_as_float(sign | 0x7F800000u);
    return f64_to_f32_rare(d);  // float subnormals, infinities and NaN: the hardware conversion
}

__device__ __forceinline__ float f64_to_f32(float f) { return f; }

__device__ __forceinline__ double f32_to_f64(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned ef = (b >> 23) & 0xFFu;
    if (ef - 1u < 254u) {  // normal: exact re-bias and shift
        const unsigned hi = (b & 0x80000000u) | ((ef + 896u) << 20) | ((b & 0x7FFFFFu) >> 3);
        const unsigned lo = b << 29;
        return __hiloint2double((int)hi, (int)lo);
    }
    if ((b & 0x7FFFFFFFu) == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);
    return f32_to_f64_rare(f);  // subnormal, infinity, NaN
}

// ------------------------------------------------------------------------------------------
// Double-FP32 arithmetic (T. J. Dekker, "A floating-point technique for extending the available
// precision", Numer. Math. 18:224-242, 1971; D. E. Knuth, TAOCP vol. 2, 4.2.2): a value held as
// hi + lo in two FP32 numbers, about 48 significant bits, on the FP32 pipe.  Used where FP32 data
// needs products and sums beyond FP32 precision without spending FP64 instructions.
struct DF {
    float hi, lo;
};
// s + e = a + b exactly (Knuth's two-sum; no ordering of |a|, |b| needed)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// acc += a b: the product is exact as p + pe (FMA), p enters hi through two-sum and the two error
// terms gather in lo (over the hundred-odd terms a thread sums, lo stays far below hi)
__device__ __forceinline__ void df_mac(DF& acc, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);
    float s, e;
    two_sum(acc.hi, p, s, e);
    acc.hi = s;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(e, pe));
}
// acc += (c.hi + c.lo) b: c.hi b exact as above, c.lo b (a 2^-24-relative term) in one rounding
__device__ __forceinline__ void df_mac(DF& acc, DF c, float b) {
    const float p = __fmul_rn(c.hi, b);
    const float pe = __fmaf_rn(c.hi, b, -p);
    float s, e;
    two_sum(acc.hi, p, s, e);
    acc.hi = s;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(e, __fmaf_rn(c.lo, b, pe)));
}
// An FP64 scalar split as hi = RN32(d), lo = RN32(d - hi) (once per thread, not per element)
__device__ __forceinline__ DF df_split(double d) {
    const float hi = __double2float_rn(d);
    return DF{hi, __double2float_rn(__dsub_rn(d, (double)hi))};
}
__device__ __forceinline__ double df_to_f64(DF a) { return __dadd_rn(f32_to_f64(a.hi), f32_to_f64(a.lo)); }

// hi + lo -= x, the rounding error of the subtraction gathered in lo (two-sum)
__device__ __forceinline__ void df_sub(float& hi, float& lo, float x) {
    float s, e;
    two_sum(hi, -x, s, e);
    hi = s;
    lo = __fadd_rn(lo, e);
}

// The Bratu3D Jacobian product h^-2 (6v - the six neighbours) - c v of FP32 values, to the accuracy of an FP32
// result, on the FP32 pipe alone: the stencil sum in double-FP32 (6v exact with its FMA error, each neighbour
// subtracted by two-sum), h^-2 s exactly as ph + pl, c v with the FP32 coefficient RN32(c) as an exact
// product (two-product), the difference in double-FP32, rounded once.  Against the product with the FP64
// coefficient this adds |c - RN32(c)| |v| <= 2^-24 |c v|, the size of the final rounding itself.
__device__ __forceinline__ float jvp32xf_point(float below, float cur, float above, float jm, float jp, float km,
                                               float kp, float c32, float h2inv) {
    float hi = __fmul_rn(6.0f, cur);
    float lo = __fmaf_rn(6.0f, cur, -hi);
    df_sub(hi, lo, below);
    df_sub(hi, lo, above);
    df_sub(hi, lo, jm);
    df_sub(hi, lo, jp);
    df_sub(hi, lo, km);
    df_sub(hi, lo, kp);
    const float ph = __fmul_rn(h2inv, hi);
    const float pl = __fmaf_rn(h2inv, lo, __fmaf_rn(h2inv, hi, -ph));
    const float q = __fmul_rn(c32, cur);
    const float qe = __fmaf_rn(c32, cur, -q);
    float s, e;
    two_sum(ph, -q, s, e);
    return __fadd_rn(s, __fadd_rn(e, __fsub_rn(pl, qe)));
}


// RN(a / b) from y = RN(1/b), for many a divided by one b (Markstein's correction): q = RN(a y) is
// within one ulp of a/b, r = a - b q is exact by FMA, and RN(q + r y) is the correctly rounded
// quotient.  That needs a, q and y well inside the normal range (r ~ 2^-52 a must not underflow):
// outside [2^-960, 2^1001) — zeros, subnormals, infinities, NaN — the IEEE division runs instead.
// Three FP64 instructions instead of a full division.
__device__ __forceinline__ unsigned fp64_biased_exp(double v) {
    return ((unsigned)__double2hiint(v) >> 20) & 0x7FFu;
}
// y for div_by_recip: RN(1/b), or 0 (every quotient then takes the IEEE division) when b is outside
// [2^-960, 2^960].
__device__ __forceinline__ double recip_for_div(double b) {
    return fp64_biased_exp(b) - 63u <= 1920u ? __ddiv_rn(1.0, b) : 0.0;
}
__device__ __forceinline__ double div_by_recip(double a, double b, double y) {
    const double q = __dmul_rn(a, y);
    const double r = __fma_rn(-q, b, a);
    const double q2 = __fma_rn(r, y, q);
    if (fp64_biased_exp(a) - 63u > 1960u || fp64_biased_exp(q2) - 63u > 1960u) return __ddiv_rn(a, b);
    return q2;
}

// ------------------------------------------------------------------------------------------
// e^x by Tang's table-driven method (P. T. P. Tang, "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2):144-157, 1989), with a
// 2048-entry table and every part that needs no FP64 moved to the FP32 and integer pipes (on this
// GPU the FP64 pipe issues about 2 instructions per clock per SM against 128 FP32 ones):
//   x = (2048 M + j) ln2/2048 + r,   e^x = 2^M * 2^(j/2048) * e^r,   |r| <= ~ln2/4096 < 1.7e-4,
// with 2^(j/2048) = T_hi + T_lo from exp2_table.cuh (gen_exp2_table.py).
//  * N = 2048 M + j = round(2048 x / ln2) is formed in FP32 from x truncated to FP32 (near a tie it
//    may be the other neighbour, which only widens |r| a little); the FP32 value N (an integer below
//    2^22 in magnitude, exact) is widened to FP64 by integer instructions.
//  * ln2/2048 = L1 + L2: r = RN(x - N L1) in FP64 (one FMA); the small part N L2 (< 3e-14) is
//    folded into the table's low word in FP32, to first order: - T_hi N L2 (1 + r).
//  * e^r - 1 = (r + r^2/2) + r^3 (1/6 + r/24) + O(r^5 < 2e-21): r + r^2/2 as one FMA with r/2
//    formed by decrementing the exponent; the cubic and quartic terms (< 1e-12) in FP32, folded into
//    the low word too (their FP32 rounding stays below 1e-19).
//  * y = T_hi + (T_hi (r + r^2/2) + [T_lo - T_hi N L2 (1 + r) + T_hi r^3 (1/6 + r/24)]) in
//    [0.99, 2.01], then 2^M by adding M to the exponent field: for |x| < 708 the result is normal.
// Four FP64 instructions; within 0.505 ulp of e^x over 24M test points (99.9 % correctly rounded).
// |x| >= 708 (overflow, results near or below the smallest normal, infinities, NaN) is left to exp().
#include "exp2_table.cuh"

// v truncated to FP32 (23 fraction bits kept); values below 2^-126 in magnitude give 0
__device__ __forceinline__ float f64_trunc_f32(double v) {
    const unsigned hi = (unsigned)__double2hiint(v), lo = (unsigned)__double2loint(v);
    const unsigned a = hi & 0x7FFFFFFFu;
    return a > 0x38000000u ? __uint_as_float((hi & 0x80000000u) | ((a - 0x38000000u) << 3) | (lo >> 29)) : 0.0f;
}

// The method above for |x| below the caller's limit, with the table given: T2[j].x = T_hi (FP64),
// TF[j] = (RN32(T_hi), RN32(T_lo)).  The table may be 2^(j/2048) itself or lambda 2^(j/2048) (then
// the result is lambda e^x, as long as it stays a normal number).
__device__ __forceinline__ double exp_tang_core(double x, const double2* __restrict__ T2,
                                                const float2* __restrict__ TF) {
    const float xf = f64_trunc_f32(x);  // |x| < 708 < 2^127: no overflow
    const float tf = __fmaf_rn(xf, kExpInvL, 0x1.8p23f);
    const int N = (int)(__float_as_uint(tf) - 0x4B400000u);  // round(2048 x / ln2), |N| < 2^22
    const float nf = __fsub_rn(tf, 0x1.8p23f);  // N exactly (|N| < 2^22)
    const unsigned nb = __float_as_uint(nf);
    const double nd = (nb & 0x7FFFFFFFu)  // N in FP64: the exact widening of nf, in integer instructions
                          ? __hiloint2double((int)((nb & 0x80000000u) | (((nb & 0x7FFFFFFFu) >> 3) + (896u << 20))),
                                             (int)(nb << 29))
                          : 0.0;
    const double r = __fma_rn(-nd, kExpL1, x);
    const int rhi = __double2hiint(r), rlo = __double2loint(r);
    const double hr = ((unsigned)rhi & 0x7FF00000u) > 0x00100000u ? __hiloint2double(rhi - 0x00100000, rlo) : 0.0;
    const double p = __fma_rn(hr, r, r);  // r + r^2/2 (r^2/2 vanishes where r/2 is taken as 0)
    const float rf = f64_trunc_f32(r);
    const float t = __fmul_rn(__fmul_rn(__fmul_rn(rf, rf), rf), __fmaf_rn(rf, 0x1.555556p-5f, 0x1.555556p-3f));
    const int jj = N & ((1 << kExpTableBits) - 1);
    const double Thi = __ldg(&T2[jj].x);
    const float2 Tf = __ldg(&TF[jj]);
    const float cf = __fmaf_rn(Tf.x, t, __fmaf_rn(-__fmul_rn(Tf.x, __fmul_rn(nf, kExpL2f)), __fadd_rn(1.0f, rf), Tf.y));
    const unsigned cb = __float_as_uint(cf);
    const double c = (cb & 0x7F800000u) ? __hiloint2double((int)((cb & 0x80000000u) | (((cb & 0x7FFFFFFFu) >> 3) + (896u << 20))),
                                                           (int)(cb << 29))
                                        : 0.0;  // exact widening; FP32 zeros and subnormals (< 1.2e-38) as 0
    const double y = __dadd_rn(Thi, __fma_rn(Thi, p, c));
    return __hiloint2double(__double2hiint(y) + (N >> kExpTableBits) * (1 << 20), __double2loint(y));
}

__device__ __forceinline__ double exp_tang(double x) {
    if (((unsigned)__double2hiint(x) & 0x7FFFFFFFu) >= 0x40862000u) return exp(x);  // |x| >= 708, inf, NaN
    return exp_tang_core(x, kExp2Frac, kExp2FracF);
}

// lambda e^x from the table scaled by lambda (T2[j] = (RN(lambda T_hi), low part), TF = their RN32),
// for lambda in [2^-10, 2^10]: one FP64 multiply fewer than lambda * exp_tang(x).  Below |x| = 690
// the result lies within [2^-1006, 2^1006], a normal number; beyond, lambda * exp(x).  The low part
// carries the rounding error of lambda T_hi, so the result is within 0.503 ulp of lambda e^x (16M
// points at each of seven lambda in a CPU restatement), where lambda * exp_tang(x) rounds twice and
// reaches 1.5 ulp.
__device__ __forceinline__ double lam_exp_tang(double x, double lam, const double2* __restrict__ T2,
                                               const float2* __restrict__ TF) {
    if (((unsigned)__double2hiint(x) & 0x7FFFFFFFu) >= 0x40859000u) return lam * exp(x);  // |x| >= 690, inf, NaN
    return exp_tang_core(x, T2, TF);
}

// ------------------------------------------------------------------------------------------
// 6c - (a1 + ... + a6) of seven FP64 values in 64-bit fixed point on the integer pipe, rounded once to
// FP64: GB300's FP64 pipe issues about two instructions a clock per SM, its integer pipe thirty-two
// times that, and the six FP64 operations of the sum were half of a residual evaluation's FP64 work.
// Each value's 53-bit significand is placed 4 bits up in a signed 64-bit integer, aligned to the
// largest exponent E of the seven (bits below 2^(E-1079) truncated: an error of at most 7 such
// units, 2^-56 of the largest value); 6c and the sum stay below 2^61; the total is normalised and
// rounded to nearest-even.  So the result is within 2^-56 |largest value| + half an ulp of the exact
// sum (the FP64 chain of six roundings: up to ~3 2^-53 of the largest partial sum).  Infinities,
// NaN and results outside the normal range go to the FP64 chain (a call that is not inlined).
static __device__ __noinline__ double lap7_fp64_rare(double c, double a1, double a2, double a3, double a4, double a5,
                                                      double a6) {
    double s = __fma_rn(6.0, c, -a1);
    s = s - a2;
    s = s - a3;
    s = s - a4;
    s = s - a5;
    return s - a6;
}
// A value's fixed-point parts: 53-bit significand (hidden bit set for normal numbers), exponent
// (1 for zeros and subnormals), sign.
struct FxParts {
    unsigned long long mag;
    int e;
    bool neg;
};
__device__ __forceinline__ FxParts fx_split(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int eb = (int)((b >> 52) & 0x7FFu);
    FxParts f;
    f.mag = (b & 0xFFFFFFFFFFFFFull) | (eb ? (1ull << 52) : 0ull);
    f.e = eb ? eb : 1;  // a subnormal: exponent 1 without the hidden bit
    f.neg = (long long)b < 0;
    return f;
}
__device__ __forceinline__ long long fx_term(const FxParts& f, int E) {
    // E - f.e >= 57 leaves nothing of the 57-bit value; 63 keeps the shift defined
    const unsigned long long t = (f.mag << 4) >> min(E - f.e, 63);
    return f.neg ? -(long long)t : (long long)t;
}
// S 2^(E - 1079) rounded to nearest-even as an FP64 value, for |S| < 2^61; false where the result would be
// subnormal (the caller's rare path).
__device__ __forceinline__ bool fx_round(long long S, int E, double& out) {
    if (S == 0) {
        out = 0.0;
        return true;
    }
    const unsigned long long sign = S < 0 ? (1ull << 63) : 0ull;
    unsigned long long A = S < 0 ? (unsigned long long)(-S) : (unsigned long long)S;
    const int lz = __clzll((long long)A);  // >= 3
    const int eb = E + 7 - lz;             // the biased exponent of A 2^(E - 1079)
    if (eb <= 0) return false;
    A <<= lz;                                   // leading one at bit 63
    unsigned long long mant = A >> 11;          // 53 bits
    const unsigned rem = (unsigned)(A & 0x7FFu);
    mant += (rem > 0x400u || (rem == 0x400u && (mant & 1ull))) ? 1ull : 0ull;
    // the hidden bit adds one to the exponent field; a carry out of the significand adds one more
    out = __longlong_as_double((long long)(sign | ((((unsigned long long)(eb - 1)) << 52) + mant)));
    return true;
}
// The sum from the seven values' parts (c first); the values themselves for the rare cases.
__device__ __forceinline__ double lap7_fixed(const FxParts& f0, const FxParts& f1, const FxParts& f2, const FxParts& f3,
                                             const FxParts& f4, const FxParts& f5, const FxParts& f6, double c,
                                             double a1, double a2, double a3, double a4, double a5, double a6) {
    const int E = max(max(max(f0.e, f1.e), max(f2.e, f3.e)), max(max(f4.e, f5.e), f6.e));
    if (E >= 2040) return lap7_fp64_rare(c, a1, a2, a3, a4, a5, a6);  // infinities, NaN, near overflow
    const long long t0 = fx_term(f0, E);
    const long long S = ((t0 << 2) + (t0 << 1)) - fx_term(f1, E) - fx_term(f2, E) - fx_term(f3, E) - fx_term(f4, E) -
                        fx_term(f5, E) - fx_term(f6, E);
    double out;
    if (!fx_round(S, E, out)) return lap7_fp64_rare(c, a1, a2, a3, a4, a5, a6);  // a subnormal result
    return out;
}

// (a1 + a2) + (a3 + a4) - 4c, the 5-point sum of a 2D Laplacian, in the same fixed point, rounded once
// (|sum| < 2^60 of the aligned units); the FP64 form of the differences for the rare cases.
static __device__ __noinline__ double lap5_fp64_rare(double c, double a1, double a2, double a3, double a4) {
    return ((a1 - c) + (a2 - c)) + ((a3 - c) + (a4 - c));
}
__device__ __forceinline__ double lap5_fixed(double c, double a1, double a2, double a3, double a4) {
    const FxParts f0 = fx_split(c), f1 = fx_split(a1), f2 = fx_split(a2), f3 = fx_split(a3), f4 = fx_split(a4);
    const int E = max(max(f0.e, f1.e), max(max(f2.e, f3.e), f4.e));
    if (E >= 2040) return lap5_fp64_rare(c, a1, a2, a3, a4);
    const long long S = (fx_term(f1, E) + fx_term(f2, E)) + (fx_term(f3, E) + fx_term(f4, E)) - (fx_term(f0, E) << 2);
    double out;
    if (!fx_round(S, E, out)) return lap5_fp64_rare(c, a1, a2, a3, a4);
    return out;
}
__device__ __forceinline__ double lap7_fixed(double c, double a1, double a2, double a3, double a4, double a5,
                                             double a6) {
    return lap7_fixed(fx_split(c), fx_split(a1), fx_split(a2), fx_split(a3), fx_split(a4), fx_split(a5),
                      fx_split(a6), c, a1, a2, a3, a4, a5, a6);
}

// ------------------------------------------------------------------------------------------
// One process-wide lock held across every CUDA-graph capture and around every device or pinned
// allocation and free: cudaFree / cudaMallocHost may synchronise the whole device, which would
// break a capture another thread (another context) has in progress.  Recursive, so a capture
// that allocated would fail in CUDA rather than deadlock here.
std::recursive_mutex& alloc_capture_mutex();

// ------------------------------------------------------------------------------------------
// Host-side context: one device, one stream, reduction scratch and device scalars.
constexpr int kNumScalars = 2048;
constexpr size_t kMaxRestart = 250;  // GMRES(m) limit of the device scalar layout below

struct Context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    RedArgs red{};
    double* d_scalars = nullptr;  // kNumScalars device scalars
    double* h_scalars = nullptr;  // pinned host mirror
    cudaEvent_t done = nullptr;
    uint64_t launches = 0;
    bool timing = false;
    std::string last_error;

    explicit Context(int dev);
    ~Context();
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;

    void sync();
    // Copies count device doubles to host memory and waits for them.
    void fetch(const double* dsrc, int count, double* host);
    double fetch1(const double* dsrc) {
        double v;
        fetch(dsrc, 1, &v);
        return v;
    }
    double* scalar(int slot) { return d_scalars + slot; }
    // Number of blocks of kRedThreads threads for a grid-stride reduction over N elements.
    unsigned red_grid(size_t N) const;
    void count_launch(unsigned n = 1) { launches += n; }
    void check_launch(const char* what);
};
// Programmatic dependent launch.  A kernel launched by launch_pdl may be scheduled while its
// predecessor on the stream is still running; it must call pdl_wait() before it touches memory
// (griddepcontrol.wait returns once every prerequisite grid has completed and its writes are
// visible).  pdl_trigger() lets this grid's own dependents be scheduled once all its CTAs have
// issued it; they still wait for its completion.  Both are no-ops in a kernel launched normally.
// In a chain of small kernels (the coarse levels of a V-cycle) this hides the launch latency
// between consecutive kernels, on a stream or inside a captured graph.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... KArgs, class... Args>
void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    NUMA_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

// Largest dynamic shared memory a block may opt in to on the context's device (bytes).
int smem_optin_limit(Context& ctx);

// Sets a kernel's dynamic shared-memory limit to the most the device allows beside the kernel's
// static shared memory, and returns it.  The attribute belongs to the kernel, not to one caller:
// a fixed value lets hierarchies and grids of any size share the kernel (a caller setting its own
// need would lower the limit under another's launch).
template <class K>
int set_dynamic_smem_limit(Context& ctx, K* kernel) {
    cudaFuncAttributes a;
    NUMA_CUDA(cudaFuncGetAttributes(&a, kernel));
    const int lim = smem_optin_limit(ctx) - (int)a.sharedSizeBytes;
    NUMA_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    return lim;
}

// Device scalar slots with fixed roles.
enum ScalarSlot : int {
    kSlotTmp0 = 0,        // public-API reductions
    kSlotTmp1 = 1,
    kSlotNormF = 8,       // ||F|| of the last evaluation
    kSlotFdH = 16,        // finite-difference step h, 1/h, zero-direction flag
    kSlotFdRh = 17,
    kSlotFdZero = 18,
    kSlotFdXnorm = 19,
    kSlotFdInvH = 20,     // RN(1/h) and RN(1/h^2) for the quotients
    kSlotFdInvHH = 21,
    kSlotPieceSums = 24,  // sums of squares of an evaluation's pieces, 8 entries
    kSlotGmresH = 64,      // Hessenberg column, m + 2 entries (m <= kMaxRestart)
    kSlotGmresH2 = 320,    // CGS2 second-pass coefficients, m + 1 entries
    kSlotGmresY = 640,     // least-squares solution y, m entries
    kSlotGmresCoef = 900,  // recycled-solve coefficients, 2k + 1 entries
    kSlotGmresSig2 = 1408, // lazily normalised basis: 1 / norm^2 of each vector, m + 1 entries
    kSlotGmresSig = 1664,  // FP32 basis: 1 / norm of each vector, m + 1 entries
};

// Pinned host staging for small vectors moving to the device.
struct PinnedBuf {
    double* p = nullptr;
    size_t cap = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() {
        if (p) {
            std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
            cudaFreeHost(p);
        }
    }
    double* get(size_t count) {
        if (count > cap) {
            std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
            if (p) cudaFreeHost(p);
            p = nullptr;
            cap = 0;
            NUMA_CUDA(cudaMallocHost(reinterpret_cast<void**>(&p), count * sizeof(double)));
            cap = count;
        }
        return p;
    }
};

// Owning device array with capacity reuse.
template <class T>
struct DeviceArray {
    T* p = nullptr;
    size_t n = 0;
    size_t cap = 0;
    DeviceArray() = default;
    explicit DeviceArray(size_t count) { resize(count); }
    ~DeviceArray() { release(); }
    DeviceArray(const DeviceArray&) = delete;
    DeviceArray& operator=(const DeviceArray&) = delete;
    DeviceArray(DeviceArray&& o) noexcept : p(o.p), n(o.n), cap(o.cap) { o.p = nullptr; o.n = o.cap = 0; }
    DeviceArray& operator=(DeviceArray&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p; n = o.n; cap = o.cap;
            o.p = nullptr; o.n = o.cap = 0;
        }
        return *this;
    }
    void resize(size_t count) {
        if (count > cap) {
            std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
            release();
            if (count > 0) {
                cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T));
                if (e == cudaErrorMemoryAllocation) {
                    cudaGetLastError();
                    p = nullptr;
                    throw Status(NUMA_GPU_ERR_OUT_OF_MEMORY, "cudaMalloc failed: out of device memory");
                }
                NUMA_CUDA(e);
            }
            cap = count;
        }
        n = count;
    }
    void release() {
        if (p) {
            std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
            cudaFree(p);
        }
        p = nullptr;
        n = cap = 0;
    }
    void swap(DeviceArray& o) noexcept {
        std::swap(p, o.p);
        std::swap(n, o.n);
        std::swap(cap, o.cap);
    }
};

}  // namespace numa::gpu

// Public opaque handle types (declared in numa_gpu.h).
struct numa_gpu_ctx {
    numa::gpu::Context* impl;
};

struct numa_gpu_vec {
    numa_gpu_ctx* ctx;
    double* d;
    size_t n;
    bool owns;
};
