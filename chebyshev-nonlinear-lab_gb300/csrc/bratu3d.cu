// bratu3d.cu — Bratu3D residual, Jacobian-vector products and second directional derivatives
// (problems/bratu3d.hpp, operators/operator.hpp:101-134) on the GPU.
//
// Layout: n^3 FP64 values, index (i*n + j)*n + k with k fastest, Dirichlet zeros implicit.
// Kernels march along i: a block covers a 32 x 8 tile of (k, j) and walks a chunk of i planes,
// keeping the i-1, i, i+1 values of its column in registers, so each point issues five loads.
// The 7-point sums follow the reference's operation order (6v, then minus the i-1, i+1, j-1,
// j+1, k-1, k+1 neighbours; a missing neighbour subtracts +0.0, which leaves every value
// unchanged), so the stencil results equal the reference's bit for bit; only e^x may differ by
// an ulp between the table-driven exp_tang (common.cuh) and the host C library.
#include <cmath>
#include <limits>
#include <type_traits>

#include "numa_internal.hpp"

namespace numa::gpu {
namespace {

constexpr int BX = 32, BY = 8;

struct March {
    dim3 grid;
    int ichunk;
};

// Grid of (k tiles, j tiles, i chunks).  Chunks of 8 planes keep ~2M threads at n = 255; a fused
// reduction takes 16 from n = 128 (its block sum, in FP64, is then shared by twice the points), and
// more when it would exceed kMaxRedBlocks partials.
March march_shape(int n, bool reducing) {
    const int kb = (n + BX - 1) / BX, jb = (n + BY - 1) / BY;
    int ichunk = n >= 64 ? (reducing && n >= 128 ? 16 : 8) : (n >= 16 ? 4 : 1);
    if (reducing) {
        const long cols = (long)kb * jb;
        const long max_chunks = kMaxRedBlocks / cols;
        if (max_chunks < 1) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "grid too large for a fused reduction");
        const long need = (n + max_chunks - 1) / max_chunks;
        if (need > ichunk) ichunk = (int)need;
    }
    March m;
    m.ichunk = ichunk;
    m.grid = dim3(kb, jb, (n + ichunk - 1) / ichunk);
    return m;
}

// Minus the 7-point Laplacian without the h^-2 factor, on a value column marching in i.
__device__ __forceinline__ double lap_sum(const double* __restrict__ v, size_t p, size_t plane, int n, int i,
                                          int j, int k, double below, double cur, double& above) {
    above = (i + 1 < n) ? v[p + plane] : 0.0;
    const double jm = (j > 0) ? v[p - n] : 0.0;
    const double jp = (j + 1 < n) ? v[p + n] : 0.0;
    const double km = (k > 0) ? v[p - 1] : 0.0;
    const double kp = (k + 1 < n) ? v[p + 1] : 0.0;
    double s = 6.0 * cur;
    s = s - below;
    s = s - above;
    s = s - jm;
    s = s - jp;
    s = s - km;
    s = s - kp;
    return s;
}

// F = h^-2 (6u - sum) - lambda e^u; optionally c = lambda e^u and ||F||.  The last step is one FMA
// (F differs from the reference's two roundings by at most half an ulp, as e^u already may).
// C32: also c32 = RN32(c) (the mixed path's FP32 Jacobian coefficient) and f32 = RN32(F) (the
// first FP32 Krylov vector of the next linear solve), integer conversions; this is the mixed
// path's evaluation, and it forms 6u - (the six neighbours) in 64-bit fixed point on the integer pipe,
// rounded once (lap7_fixed; the reference rounds six times).  LT: lambda e^u from the operator's
// lambda-scaled exp table (lt2, ltf).  The C32 form is held to five resident CTAs an SM (48 registers):
// its integer and FP64 pipes are both busy, and the extra warps cover more of their latency.
template <bool WRITE_C, bool NORM, bool C32, bool LT>
__global__ void __launch_bounds__(BX* BY, C32 ? 5 : 1) k_eval(const double* __restrict__ u, double* __restrict__ F,
                                                 double* __restrict__ c_out, float* __restrict__ c32_out,
                                                 float* __restrict__ f32_out, int n,
                                                 int ichunk, double lam, double h2inv, RedArgs red, double* norm_out,
                                                 int zoff, int norm_raw, const double2* __restrict__ lt2,
                                                 const float2* __restrict__ ltf) {
    pdl_wait();
    pdl_trigger();
    const int k = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int i0 = (blockIdx.z + zoff) * ichunk;  // zoff: the first plane chunk of a piece
    const int i1 = min(i0 + ichunk, n);
    const size_t plane = (size_t)n * n;
    double acc[1] = {0.0};
    if (k < n && j < n) {
        size_t p = ((size_t)i0 * n + j) * n + k;
        double below = (i0 > 0) ? u[p - plane] : 0.0;
        double cur = u[p];
        // the mixed path's fixed-point parts of the column values, split once and carried along i
        FxParts fb{}, fc{};
        if (C32) {
            fb = fx_split(below);
            fc = fx_split(cur);
        }
        for (int i = i0; i < i1; ++i) {
            double above;
            double s;
            if (C32) {
                above = (i + 1 < n) ? u[p + plane] : 0.0;
                const double jm = (j > 0) ? u[p - n] : 0.0;
                const double jp = (j + 1 < n) ? u[p + n] : 0.0;
                const double km = (k > 0) ? u[p - 1] : 0.0;
                const double kp = (k + 1 < n) ? u[p + 1] : 0.0;
                const FxParts fa = fx_split(above);
                s = lap7_fixed(fc, fb, fa, fx_split(jm), fx_split(jp), fx_split(km), fx_split(kp), cur, below, above,
                               jm, jp, km, kp);
                fb = fc;
                fc = fa;
            } else {
                s = lap_sum(u, p, plane, n, i, j, k, below, cur, above);
            }
            const double e = LT ? lam_exp_tang(cur, lam, lt2, ltf) : lam * exp_tang(cur);
            const double f = __fma_rn(h2inv, s, -e);  // h^-2 s - e with one rounding
            F[p] = f;
            if (WRITE_C) c_out[p] = e;
            if (C32) {
                c32_out[p] = f64_to_f32(e);
                f32_out[p] = f64_to_f32(f);
            }
            if (NORM) acc[0] = __fma_rn(f, f, acc[0]);
            below = cur;
            cur = above;
            p += plane;
        }
    }
    if (NORM) {
        __shared__ double sm[1][32];
        block_sum<1>(acc, sm);
        grid_reduce_finish<1>(acc, red, [norm_out, norm_raw] __device__(const double(&t)[1]) {
            *norm_out = norm_raw ? t[0] : __dsqrt_rn(t[0]);  // raw: a piece's sum of squares
        });
    }
}

// The exp table scaled by lambda: T2[j] = (RN(lambda T_hi), lambda T_hi - RN(lambda T_hi) + lambda T_lo),
// TF[j] = RN32 of both (the unscaled table is 2^(j/2048) = T_hi + T_lo).
__global__ void k_lam_table(double lam, double2* __restrict__ T2, float2* __restrict__ TF) {
    const int jj = blockIdx.x * blockDim.x + threadIdx.x;
    if (jj >= (1 << kExpTableBits)) return;
    const double2 T = kExp2Frac[jj];
    const double hi = __dmul_rn(lam, T.x);
    const double lo = __dadd_rn(__fma_rn(lam, T.x, -hi), __dmul_rn(lam, T.y));
    T2[jj] = make_double2(hi, lo);
    TF[jj] = make_float2(__double2float_rn(hi), __double2float_rn(lo));
}

// c = lambda e^u
__global__ void k_coef(const double* __restrict__ u, double* __restrict__ c, size_t N, double lam) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) c[p] = lam * exp_tang(u[p]);
}

// out = h^-2 (6v - sum) - c v, with c given (FROM_X: c = lambda e^x formed here).
template <bool FROM_X>
__global__ void __launch_bounds__(BX* BY) k_jvp(const double* __restrict__ cx, const double* __restrict__ v,
                                                double* __restrict__ out, int n, int ichunk, double lam,
                                                double h2inv) {
    pdl_wait();
    pdl_trigger();
    const int k = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int i0 = blockIdx.z * ichunk;
    const int i1 = min(i0 + ichunk, n);
    if (k >= n || j >= n) return;
    const size_t plane = (size_t)n * n;
    size_t p = ((size_t)i0 * n + j) * n + k;
    double below = (i0 > 0) ? v[p - plane] : 0.0;
    double cur = v[p];
    for (int i = i0; i < i1; ++i) {
        double above;
        const double s = lap_sum(v, p, plane, n, i, j, k, below, cur, above);
        const double c = FROM_X ? lam * exp_tang(cx[p]) : cx[p];
        out[p] = h2inv * s - c * cur;
        below = cur;
        cur = above;
        p += plane;
    }
}

// Mixed precision: F'(x) v in FP32 arithmetic on FP64 vectors with an FP32 coefficient.  Each
// FP64 value is converted once (integer arithmetic, no FP64 instruction) into a shared-memory
// plane of the tile with a 1-point halo; three plane slots roll along i.  Software-pipelined:
// the raw values of plane i+2 and the coefficient of plane i+1 are loaded into registers while
// plane i is computed, so the loads' latency overlaps the arithmetic.
__device__ __forceinline__ float to_f32(double x) { return f64_to_f32(x); }
__device__ __forceinline__ float to_f32(float x) { return x; }

template <class VT>
__global__ void __launch_bounds__(BX* BY) k_jvp32(const float* __restrict__ c32, const VT* __restrict__ v,
                                                  double* __restrict__ out, int n, int ichunk, float h2inv) {
    pdl_wait();
    pdl_trigger();
    constexpr int TW = BX + 2, TH = BY + 2, TE = TW * TH;  // 34 x 10 tile, 340 values
    constexpr int PER = (TE + BX * BY - 1) / (BX * BY);    // values per thread and plane (2)
    __shared__ float S[3][TH][TW];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * BX + tx;
    const int k0 = blockIdx.x * BX, j0 = blockIdx.y * BY;
    const int k = k0 + tx, j = j0 + ty;
    const int i0 = blockIdx.z * ichunk;
    const int i1 = min(i0 + ichunk, n);
    const size_t plane = (size_t)n * n;
    // this thread's tile elements: offset within a plane (or -1 outside the grid) and position
    int off[PER], pos[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int e = tid + q * BX * BY;
        const int r = e / TW, cc = e - r * TW;
        const int jj = j0 - 1 + r, kk = k0 - 1 + cc;
        pos[q] = e < TE ? e : -1;
        off[q] = (e < TE && jj >= 0 && jj < n && kk >= 0 && kk < n) ? jj * n + kk : -1;
    }
    VT raw[PER];
    auto issue = [&](int p) {
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            raw[q] = VT(0);
            if (p >= 0 && p < n && off[q] >= 0) raw[q] = v[(size_t)p * plane + off[q]];
        }
    };
    auto commit = [&](int p) {
        float* T = &S[(p + 3) % 3][0][0];
#pragma unroll
        for (int q = 0; q < PER; ++q)
            if (pos[q] >= 0) T[pos[q]] = to_f32(raw[q]);
    };
    const bool inside = k < n && j < n;
    const size_t col = (size_t)j * n + k;
    issue(i0 - 1);
    commit(i0 - 1);
    issue(i0);
    commit(i0);
    issue(i0 + 1);
    float cnext = (inside && i0 < i1) ? c32[(size_t)i0 * plane + col] : 0.0f;
    for (int i = i0; i < i1; ++i) {
        commit(i + 1);
        if (i + 2 <= i1) issue(i + 2);
        const float cc = cnext;
        if (inside && i + 1 < i1) cnext = c32[(size_t)(i + 1) * plane + col];
        __syncthreads();
        if (inside) {
            const float(*Tm)[TW] = S[(i + 2) % 3];
            const float(*T0)[TW] = S[i % 3];
            const float(*Tp)[TW] = S[(i + 1) % 3];
            const float cur = T0[ty + 1][tx + 1];
            float s = 6.0f * cur;
            s = s - Tm[ty + 1][tx + 1];
            s = s - Tp[ty + 1][tx + 1];
            s = s - T0[ty][tx + 1];
            s = s - T0[ty + 2][tx + 1];
            s = s - T0[ty + 1][tx];
            s = s - T0[ty + 1][tx + 2];
            out[(size_t)i * plane + col] = f32_to_f64(h2inv * s - cc * cur);
        }
        __syncthreads();
    }
}

// One point of k_jvp32f: h^-2 (6 v - the six neighbours, i-1, i+1, j-1, j+1, k-1, k+1) - c v.
__device__ __forceinline__ float jvp32_point(float below, float cur, float above, float jm, float jp, float km,
                                             float kp, float cc, float h2inv) {
    float s = 6.0f * cur;
    s = s - below;
    s = s - above;
    s = s - jm;
    s = s - jp;
    s = s - km;
    s = s - kp;
    return h2inv * s - cc * cur;
}

template <class OT>
__device__ __forceinline__ void jvp32_store(OT* __restrict__ out, size_t p, float r) {
    if constexpr (sizeof(OT) == 4) out[p] = r;
    else out[p] = f32_to_f64(r);
}

// The FP32 product from an FP32 v (the V-cycle's output): no conversion, so no shared-memory tile —
// a (k, j) column marches in i holding planes i-1, i, i+1 in registers, and the neighbours in j and k
// come through L1.  The arithmetic is k_jvp32's, operation for operation (same results); OT = float
// stores the FP32 result as it is, OT = double widens it.
template <class OT>
__global__ void __launch_bounds__(BX* BY) k_jvp32f(const float* __restrict__ c32, const float* __restrict__ v,
                                                   OT* __restrict__ out, int n, int ichunk, float h2inv) {
    pdl_wait();
    pdl_trigger();
    const int k = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    if (k >= n || j >= n) return;
    const int i0 = blockIdx.z * ichunk;
    const int i1 = min(i0 + ichunk, n);
    const size_t plane = (size_t)n * n;
    const size_t col = (size_t)j * n + k;
    const bool jlo = j > 0, jhi = j + 1 < n, klo = k > 0, khi = k + 1 < n;
    float below = i0 > 0 ? v[(size_t)(i0 - 1) * plane + col] : 0.0f;
    float cur = i0 < i1 ? v[(size_t)i0 * plane + col] : 0.0f;
    int i = i0;
    // two planes a step, all their loads issued before either store: twice the bytes in flight
    for (; i + 1 < i1; i += 2) {
        const size_t p = (size_t)i * plane + col, q = p + plane;
        const float a1 = v[q];  // i + 1 < i1 <= n
        const float a2 = (i + 2 < n) ? v[q + plane] : 0.0f;
        const float jm0 = jlo ? v[p - n] : 0.0f, jp0 = jhi ? v[p + n] : 0.0f;
        const float km0 = klo ? v[p - 1] : 0.0f, kp0 = khi ? v[p + 1] : 0.0f;
        const float jm1 = jlo ? v[q - n] : 0.0f, jp1 = jhi ? v[q + n] : 0.0f;
        const float km1 = klo ? v[q - 1] : 0.0f, kp1 = khi ? v[q + 1] : 0.0f;
        const float c0 = c32[p], c1 = c32[q];
        jvp32_store(out, p, jvp32_point(below, cur, a1, jm0, jp0, km0, kp0, c0, h2inv));
        jvp32_store(out, q, jvp32_point(cur, a1, a2, jm1, jp1, km1, kp1, c1, h2inv));
        below = a1;
        cur = a2;
    }
    if (i < i1) {
        const size_t p = (size_t)i * plane + col;
        const float above = (i + 1 < n) ? v[p + plane] : 0.0f;
        const float jm = jlo ? v[p - n] : 0.0f, jp = jhi ? v[p + n] : 0.0f;
        const float km = klo ? v[p - 1] : 0.0f, kp = khi ? v[p + 1] : 0.0f;
        jvp32_store(out, p, jvp32_point(below, cur, above, jm, jp, km, kp, c32[p], h2inv));
    }
}

// One point of k_jvp32x: the product from FP32 values to FP64 accuracy on the FP32 pipe.  The
// Laplacian sum 6v - (six neighbours) in double-FP32 arithmetic: 6v exact as a product and its FMA
// error, each neighbour subtracted by two-sum with the rounding errors gathered in lo; scaled by
// h^-2 (an FP32 integer below 2^24, so h^-2 hi is exact with its FMA error); widened to FP64 in one
// addition; out = T - c v in one FP64 FMA with the FP64 coefficient.  Two FP64 instructions a point
// (the FP64 product takes ten), and an error of a few 2^-48 of the largest partial sum.
__device__ __forceinline__ double jvp32x_point(float below, float cur, float above, float jm, float jp, float km,
                                               float kp, double c, float h2inv) {
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
    const double t = __dadd_rn(f32_to_f64(ph), f32_to_f64(pl));
    return __fma_rn(-c, f32_to_f64(cur), t);
}

// FP32 out: the coefficient array is RN32(c) and jvp32xf_point forms the result (no FP64 instruction).
// FP64 out: the FP64 coefficient and jvp32x_point.
template <class OT, class CT>
__device__ __forceinline__ OT jvp32x_any(float below, float cur, float above, float jm, float jp, float km, float kp,
                                         CT c, float h2inv) {
    if constexpr (sizeof(OT) == 4) return jvp32xf_point(below, cur, above, jm, jp, km, kp, c, h2inv);
    else return jvp32x_point(below, cur, above, jm, jp, km, kp, c, h2inv);
}

// The bound product from an FP32 v (the V-cycle's output) for Krylov solves whose tolerance is below
// what FP32 arithmetic reaches: FP64 out with the FP64 coefficient, or FP32 out with RN32(c).  Same
// march as k_jvp32f: a (k, j) column walks i two planes a step with planes i-1, i, i+1 in registers.
template <class OT>
__global__ void __launch_bounds__(BX* BY) k_jvp32x(const std::conditional_t<sizeof(OT) == 4, float, double>* __restrict__ c,
                                                   const float* __restrict__ v, OT* __restrict__ out, int n, int ichunk,
                                                   float h2inv) {
    pdl_wait();
    pdl_trigger();
    const int k = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    if (k >= n || j >= n) return;
    const int i0 = blockIdx.z * ichunk;
    const int i1 = min(i0 + ichunk, n);
    const size_t plane = (size_t)n * n;
    const size_t col = (size_t)j * n + k;
    const bool jlo = j > 0, jhi = j + 1 < n, klo = k > 0, khi = k + 1 < n;
    float below = i0 > 0 ? v[(size_t)(i0 - 1) * plane + col] : 0.0f;
    float cur = i0 < i1 ? v[(size_t)i0 * plane + col] : 0.0f;
    int i = i0;
    for (; i + 1 < i1; i += 2) {
        const size_t p = (size_t)i * plane + col, q = p + plane;
        const float a1 = v[q];  // i + 1 < i1 <= n
        const float a2 = (i + 2 < n) ? v[q + plane] : 0.0f;
        const float jm0 = jlo ? v[p - n] : 0.0f, jp0 = jhi ? v[p + n] : 0.0f;
        const float km0 = klo ? v[p - 1] : 0.0f, kp0 = khi ? v[p + 1] : 0.0f;
        const float jm1 = jlo ? v[q - n] : 0.0f, jp1 = jhi ? v[q + n] : 0.0f;
        const float km1 = klo ? v[q - 1] : 0.0f, kp1 = khi ? v[q + 1] : 0.0f;
        const auto c0 = c[p], c1 = c[q];
        out[p] = jvp32x_any<OT>(below, cur, a1, jm0, jp0, km0, kp0, c0, h2inv);
        out[q] = jvp32x_any<OT>(cur, a1, a2, jm1, jp1, km1, kp1, c1, h2inv);
        below = a1;
        cur = a2;
    }
    if (i < i1) {
        const size_t p = (size_t)i * plane + col;
        const float above = (i + 1 < n) ? v[p + plane] : 0.0f;
        const float jm = jlo ? v[p - n] : 0.0f, jp = jhi ? v[p + n] : 0.0f;
        const float km = klo ? v[p - 1] : 0.0f, kp = khi ? v[p + 1] : 0.0f;
        out[p] = jvp32x_any<OT>(below, cur, above, jm, jp, km, kp, c[p], h2inv);
    }
}

// c32 = RN32(c) (integer conversion)
__global__ void k_coef32(const double* __restrict__ c, float* __restrict__ c32, size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) c32[i] = f64_to_f32(c[i]);
}

// out = -c v v  (bratu3d.hpp:52: -lambda * exp(u) * v * v, evaluated left to right)
__global__ void k_d2(const double* __restrict__ c, const double* __restrict__ v, double* __restrict__ out, size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) {
        const double vv = v[p];
        out[p] = ((-c[p]) * vv) * vv;
    }
}

// d = 6 h^-2 - c
__global__ void k_jacobi_diag(const double* __restrict__ c, double* __restrict__ d, size_t N, double six_h2inv) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) d[p] = six_h2inv - c[p];
}

unsigned ew_grid(const Context& ctx, size_t N) {
    size_t want = (N + 255) / 256;
    size_t cap = static_cast<size_t>(ctx.sm_count) * 16;
    if (want > cap) want = cap;
    return static_cast<unsigned>(want < 1 ? 1 : want);
}

}  // namespace

Bratu3D::Bratu3D(Context& ctx, size_t n, double lambda)
    : NonlinearOp(ctx), n_(n), N_(n * n * n), lambda_(lambda), h2inv_((n + 1.0) * (n + 1.0)) {
    if (n == 0) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "Bratu3D needs n > 0");
    if (n > 65535 * 8) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "grid too large");
    set_lambda(lambda);
}

// lambda in [2^-10, 2^10]: the evaluation takes lambda e^u from a table scaled by lambda (one FP64
// multiply a point fewer); otherwise lambda * e^u.
void Bratu3D::set_lambda(double lambda) {
    lambda_ = lambda;
    lt_on_ = lambda >= 0x1p-10 && lambda <= 0x1p10;
    if (!lt_on_) return;
    lt2_.resize(1 << kExpTableBits);
    ltf_.resize(1 << kExpTableBits);
    k_lam_table<<<(1 << kExpTableBits) / 256, 256, 0, ctx_.stream>>>(lambda, lt2_.p, ltf_.p);
    ctx_.count_launch();
    ctx_.check_launch("bratu3d lambda table");
}

Bratu3D::~Bratu3D() = default;

void Bratu3D::bind(const double*, const double* cache, int precision) {
    bound_c_ = cache;
    bound_precision_ = precision;
    if (precision == NUMA_GPU_FP32) {
        if (mixed_cache_) {
            bound_c32_ = reinterpret_cast<const float*>(cache + N_);  // written by the evaluation
        } else {
            c32_.resize(N_);
            coef32(cache, c32_.p);
            bound_c32_ = c32_.p;
        }
    }
}

void Bratu3D::jvp_bound32(const float* v32, double* out) {
    if (bound_precision_ != NUMA_GPU_FP32) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "Bratu3D: no FP32 product bound");
    March m = march_shape((int)n_, false);
    launch_pdl(k_jvp32f<double>, m.grid, dim3(BX, BY), 0, ctx_.stream, bound_c32_, v32, out, (int)n_, m.ichunk,
               (float)h2inv_);
    ctx_.count_launch();
    ctx_.check_launch("bratu3d jvp32 (fp32 input)");
}

void Bratu3D::jvp_bound32f(const float* v32, float* out32) {
    if (bound_precision_ != NUMA_GPU_FP32) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "Bratu3D: no FP32 product bound");
    March m = march_shape((int)n_, false);
    launch_pdl(k_jvp32f<float>, m.grid, dim3(BX, BY), 0, ctx_.stream, bound_c32_, v32, out32, (int)n_, m.ichunk,
               (float)h2inv_);
    ctx_.count_launch();
    ctx_.check_launch("bratu3d jvp32 (fp32 input and output)");
}

void Bratu3D::jvp_bound32x(const float* v32, double* out) {
    if (!has_jvp32x()) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "Bratu3D: no FP32-input FP64-accuracy product bound");
    jvp_c32x(bound_c_, v32, out);
}

void Bratu3D::jvp_c32x(const double* c, const float* v32, double* out) {
    if (n_ >= 4095) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "Bratu3D: the double-FP32 product needs n < 4095");
    March m = march_shape((int)n_, false);
    launch_pdl(k_jvp32x<double>, m.grid, dim3(BX, BY), 0, ctx_.stream, c, v32, out, (int)n_, m.ichunk,
               (float)h2inv_);
    ctx_.count_launch();
    ctx_.check_launch("bratu3d jvp32x (fp32 input, fp64 accuracy)");
}

void Bratu3D::jvp_bound32xf(const float* v32, float* out32) {
    if (!has_jvp32x()) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "Bratu3D: no FP32-input FP64-accuracy product bound");
    March m = march_shape((int)n_, false);
    launch_pdl(k_jvp32x<float>, m.grid, dim3(BX, BY), 0, ctx_.stream, bound_c32_, v32, out32, (int)n_, m.ichunk,
               (float)h2inv_);
    ctx_.count_launch();
    ctx_.check_launch("bratu3d jvp32x (fp32 input, fp64 accuracy, rounded to fp32)");
}

void Bratu3D::jvp_bound(const double* v, double* out) {
    if (bound_precision_ == NUMA_GPU_FP32) jvp_c32(bound_c32_, v, out);
    else jvp_c(bound_c_, v, out);
}

void Bratu3D::eval(const double* x, double* out, double* c_out, double* norm_out) {
    const March m = march_shape((int)n_, norm_out != nullptr);
    eval_launch(x, out, c_out, norm_out, m.grid, m.ichunk, 0, 0);
}

void Bratu3D::eval_as(const double* x, int precision, double* out, double* norm_host) {
    const bool keep = mixed_cache_;
    prepare_cache(precision);
    DeviceArray<double> cache(cache_size());
    double* nrm = ctx_.scalar(kSlotTmp0);
    eval(x, out, cache.p, nrm);
    const double v = ctx_.fetch1(nrm);
    if (norm_host) *norm_host = v;
    mixed_cache_ = keep;
}

double Bratu3D::time_eval(const double* x, int precision, int reps) {
    const bool keep = mixed_cache_;
    prepare_cache(precision);
    DeviceArray<double> out(N_), cache(cache_size());
    double* nrm = ctx_.scalar(kSlotTmp0);
    cudaEvent_t a, b;
    NUMA_CUDA(cudaEventCreate(&a));
    NUMA_CUDA(cudaEventCreate(&b));
    eval(x, out.p, cache.p, nrm);
    NUMA_CUDA(cudaEventRecord(a, ctx_.stream));
    for (int r = 0; r < reps; ++r) eval(x, out.p, cache.p, nrm);
    NUMA_CUDA(cudaEventRecord(b, ctx_.stream));
    NUMA_CUDA(cudaEventSynchronize(b));
    float ms = 0.f;
    NUMA_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    mixed_cache_ = keep;
    return reps > 0 ? ms / reps : 0.0;
}

// One launch of k_eval over the plane chunks [zoff, zoff + grid.z) (of ichunk planes each).
void Bratu3D::eval_launch(const double* x, double* out, double* c_out, double* norm_out, dim3 grid, int ichunk,
                          int zoff, int norm_raw) {
    const int n = (int)n_;
    const bool norm = norm_out != nullptr;
    const dim3 blk(BX, BY);
    float* c32 = (c_out && mixed_cache_) ? reinterpret_cast<float*>(c_out + N_) : nullptr;
    float* f32 = c32 ? reinterpret_cast<float*>(c_out + N_ + (N_ + 1) / 2) : nullptr;
    const double lam = lambda_, h2 = h2inv_;
    const RedArgs red = ctx_.red;
    const double2* t2 = lt_on_ ? lt2_.p : nullptr;
    const float2* tf = lt_on_ ? ltf_.p : nullptr;
    auto go = [&](auto kernel, double* c, float* c32v, float* f32v, double* nrm) {
        launch_pdl(kernel, grid, blk, 0, ctx_.stream, x, out, c, c32v, f32v, n, ichunk, lam, h2, red, nrm, zoff, norm_raw,
                   t2, tf);
    };
    if (lt_on_) {
        if (c32 && norm) go(k_eval<true, true, true, true>, c_out, c32, f32, norm_out);
        else if (c32) go(k_eval<true, false, true, true>, c_out, c32, f32, nullptr);
        else if (c_out && norm) go(k_eval<true, true, false, true>, c_out, nullptr, nullptr, norm_out);
        else if (c_out) go(k_eval<true, false, false, true>, c_out, nullptr, nullptr, nullptr);
        else if (norm) go(k_eval<false, true, false, true>, nullptr, nullptr, nullptr, norm_out);
        else go(k_eval<false, false, false, true>, nullptr, nullptr, nullptr, nullptr);
    } else {
        if (c32 && norm) go(k_eval<true, true, true, false>, c_out, c32, f32, norm_out);
        else if (c32) go(k_eval<true, false, true, false>, c_out, c32, f32, nullptr);
        else if (c_out && norm) go(k_eval<true, true, false, false>, c_out, nullptr, nullptr, norm_out);
        else if (c_out) go(k_eval<true, false, false, false>, c_out, nullptr, nullptr, nullptr);
        else if (norm) go(k_eval<false, true, false, false>, nullptr, nullptr, nullptr, norm_out);
        else go(k_eval<false, false, false, false>, nullptr, nullptr, nullptr, nullptr);
    }
    ctx_.count_launch();
    ctx_.check_launch("bratu3d eval");
}

// Pieces of the evaluation for an upload that overlaps it: the plane chunks of the fused-norm grid
// shared out into up to kEvalPieces runs of whole chunks.
int Bratu3D::eval_pieces() const {
    const March m = march_shape((int)n_, true);
    return (int)std::min<unsigned>(kEvalPieces, m.grid.z);
}

size_t Bratu3D::eval_piece_begin(int c) const {
    const March m = march_shape((int)n_, true);
    const int K = eval_pieces();
    const size_t plane0 = std::min<size_t>((size_t)(c * (int)m.grid.z / K) * m.ichunk, n_);
    return plane0 * n_ * n_;
}

size_t Bratu3D::eval_piece_need(int c) const {
    const March m = march_shape((int)n_, true);
    const int K = eval_pieces();
    const size_t plane1 = std::min<size_t>((size_t)((c + 1) * (int)m.grid.z / K) * m.ichunk, n_);
    return std::min(plane1 + 1, n_) * n_ * n_;  // its planes and the next one (the stencil's i + 1)
}

void Bratu3D::eval_piece(const double* x, double* out, double* cache, int c, double* sumsq) {
    const March m = march_shape((int)n_, true);
    const int K = eval_pieces();
    const int z0 = c * (int)m.grid.z / K, z1 = (c + 1) * (int)m.grid.z / K;
    eval_launch(x, out, cache, sumsq, dim3(m.grid.x, m.grid.y, (unsigned)(z1 - z0)), m.ichunk, z0, 1);
}

void Bratu3D::coef(const double* x, double* c) {
    launch_pdl(k_coef, ew_grid(ctx_, N_), 256, 0, ctx_.stream, x, c, N_, lambda_);
    ctx_.count_launch();
    ctx_.check_launch("bratu3d coef");
}

void Bratu3D::jvp_c(const double* c, const double* v, double* out) {
    March m = march_shape((int)n_, false);
    launch_pdl(k_jvp<false>, m.grid, dim3(BX, BY), 0, ctx_.stream, c, v, out, (int)n_, m.ichunk, lambda_, h2inv_);
    ctx_.count_launch();
    ctx_.check_launch("bratu3d jvp");
}

void Bratu3D::jvp_c32(const float* c32, const double* v, double* out) {
    March m = march_shape((int)n_, false);
    launch_pdl(k_jvp32<double>, m.grid, dim3(BX, BY), 0, ctx_.stream, c32, v, out, (int)n_, m.ichunk, (float)h2inv_);
    ctx_.count_launch();
    ctx_.check_launch("bratu3d jvp32");
}

// The FP32 Jacobian product of Bratu3D(n) with a given FP32 coefficient, and RN32(c), for callers
// that hold the coefficient themselves (the learned preconditioner).
void bratu_jvp32(Context& ctx, int n, double h2inv, const float* c32, const double* v, double* out) {
    March m = march_shape(n, false);
    launch_pdl(k_jvp32<double>, m.grid, dim3(BX, BY), 0, ctx.stream, c32, v, out, n, m.ichunk, (float)h2inv);
    ctx.count_launch();
    ctx.check_launch("bratu jvp32");
}

void bratu_coef32(Context& ctx, const double* c, float* c32, size_t N) {
    launch_pdl(k_coef32, ew_grid(ctx, N), 256, 0, ctx.stream, c, c32, N);
    ctx.count_launch();
}

void Bratu3D::coef32(const double* c, float* c32) {
    launch_pdl(k_coef32, ew_grid(ctx_, N_), 256, 0, ctx_.stream, c, c32, N_);
    ctx_.count_launch();
    ctx_.check_launch("bratu3d coef32");
}

void Bratu3D::jvp_x(const double* x, const double* v, double* out) {
    March m = march_shape((int)n_, false);
    launch_pdl(k_jvp<true>, m.grid, dim3(BX, BY), 0, ctx_.stream, x, v, out, (int)n_, m.ichunk, lambda_, h2inv_);
    ctx_.count_launch();
    ctx_.check_launch("bratu3d jvp(x)");
}

void Bratu3D::d2_c(const double* c, const double* v, double* out) {
    launch_pdl(k_d2, ew_grid(ctx_, N_), 256, 0, ctx_.stream, c, v, out, N_);
    ctx_.count_launch();
    ctx_.check_launch("bratu3d d2");
}

void Bratu3D::jacobi_diag_c(const double* c, double* d) {
    launch_pdl(k_jacobi_diag, ew_grid(ctx_, N_), 256, 0, ctx_.stream, c, d, N_, 6.0 * h2inv_);
    ctx_.count_launch();
    ctx_.check_launch("bratu3d jacobi_diag");
}

}  // namespace numa::gpu
