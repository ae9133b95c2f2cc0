// brusselator.cu — the Brusselator family on the GPU.
//
// * Brusselator1D: the reference's Brusselator1DStep (problems/brusselator1d.hpp:22-192), one
//   implicit-Euler step of the 1D reaction-diffusion system with Dirichlet u = 1, v = 3, and its
//   point-block Jacobi preconditioner BrusselatorJacobi (:194-222).  Every expression follows the
//   reference's order of operations (the library is compiled without FMA contraction), so F, J v,
//   F'' and the block solves are bit-identical to the reference.
// * Brusselator2D: the same reaction terms with parameters A, B, D_u, D_v, dt on an n x n periodic
//   grid of the unit square (h = 1/n), the 2-species reaction-diffusion configuration; and
//   BrussMG2D, a geometric multigrid for the coupled 2x2-block Jacobian K(w) - diag(D_u, D_v) Lap_h,
//   in FP64 (bit-identical to the CPU restatement) or FP32.
//
// Layouts.  Operator vectors are the reference's: w = (u, v) component-major, each plane
// row-major (i * n + j).  Inside BrussMG2D every level keeps (u, v) interleaved per point (one
// 8-byte FP32 or 16-byte FP64 pair) and the 2x2 block (k11, k12, k21, k22) per point (16 or 32
// bytes), so a point-block update is one vector load of each; the points are stored colour-split
// (each colour's points together, row-major), so a colour pass reads and writes only the cache
// lines of the colours it touches.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "numa_internal.hpp"

namespace numa::gpu {

namespace {

// ============================================================================== Brusselator1D
struct B1Geom {
    int n;
    double invdt, h2inv, alpha, A, B, base;
};

// F(w) (brusselator1d.hpp:47-69): boundary values u = 1, v = 3 outside the grid.
__global__ void __launch_bounds__(256) k_b1_eval(const double* __restrict__ w, const double* __restrict__ prev,
                                                 double* __restrict__ out, B1Geom G) {
    pdl_wait();
    pdl_trigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = G.n;
    if (i >= n) return;
    const double u = w[i], v = w[n + i];
    const double um = i > 0 ? w[i - 1] : 1.0, up = i + 1 < n ? w[i + 1] : 1.0;
    const double vm = i > 0 ? w[n + i - 1] : 3.0, vp = i + 1 < n ? w[n + i + 1] : 3.0;
    const double lu = (um - 2.0 * u + up) * G.h2inv;
    const double lv = (vm - 2.0 * v + vp) * G.h2inv;
    out[i] = (u - prev[i]) * G.invdt - G.alpha * lu - G.A - u * u * v + (G.B + 1.0) * u;
    out[n + i] = (v - prev[n + i]) * G.invdt - G.alpha * lv - G.B * u + u * u * v;
}

// F'(w) d (:71-98): a direction is zero outside the grid.
__global__ void __launch_bounds__(256) k_b1_jvp(const double* __restrict__ w, const double* __restrict__ d,
                                                double* __restrict__ out, B1Geom G) {
    pdl_wait();
    pdl_trigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = G.n;
    if (i >= n) return;
    const double u = w[i], v = w[n + i], du = d[i], dv = d[n + i];
    const double dum = i > 0 ? d[i - 1] : 0.0, dup = i + 1 < n ? d[i + 1] : 0.0;
    const double dvm = i > 0 ? d[n + i - 1] : 0.0, dvp = i + 1 < n ? d[n + i + 1] : 0.0;
    const double ldu = (dum - 2.0 * du + dup) * G.h2inv;
    const double ldv = (dvm - 2.0 * dv + dvp) * G.h2inv;
    out[i] = G.invdt * du - G.alpha * ldu - (2.0 * u * v) * du - u * u * dv + (G.B + 1.0) * du;
    out[n + i] = G.invdt * dv - G.alpha * ldv - G.B * du + (2.0 * u * v) * du + u * u * dv;
}

// F''(w)[d, d] = (-q, q), q = 2 v du^2 + 4 u du dv (:100-118).  Also the 2D operator's (any plane size).
__global__ void __launch_bounds__(256) k_bruss_d2(const double* __restrict__ w, const double* __restrict__ d,
                                                  double* __restrict__ out, size_t m) {
    pdl_wait();
    pdl_trigger();
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const double u = w[i], v = w[m + i], du = d[i], dv = d[m + i];
    const double q = 2.0 * v * du * du + 4.0 * u * du * dv;
    out[i] = -q;
    out[m + i] = q;
}

// The 2x2 point blocks without the off-diagonal diffusion (:120-141), one plane each.
__global__ void __launch_bounds__(256) k_b1_blocks(const double* __restrict__ w, double* __restrict__ a, B1Geom G) {
    pdl_wait();
    pdl_trigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = G.n;
    if (i >= n) return;
    const double u = w[i], v = w[n + i];
    a[i] = G.base - 2.0 * u * v + (G.B + 1.0);
    a[n + i] = -u * u;
    a[2 * n + i] = -G.B + 2.0 * u * v;
    a[3 * n + i] = G.base + u * u;
}

// BrusselatorJacobi::Bound (:198-214): z = block^-1 r, or z = r where the determinant is not
// finite or below 1e-14 in magnitude.
__global__ void __launch_bounds__(256) k_b1_block_apply(const double* __restrict__ a, const double* __restrict__ r,
                                                        double* __restrict__ z, int n) {
    pdl_wait();
    pdl_trigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a11 = a[i], a12 = a[n + i], a21 = a[2 * n + i], a22 = a[3 * n + i];
    const double ru = r[i], rv = r[n + i];
    const double det = a11 * a22 - a12 * a21;
    if (!isfinite(det) || fabs(det) < 1e-14) {
        z[i] = ru;
        z[n + i] = rv;
        return;
    }
    z[i] = (a22 * ru - a12 * rv) / det;
    z[n + i] = (-a21 * ru + a11 * rv) / det;
}

// ============================================================================== Brusselator2D
struct B2Geom {
    int n;
    double invdt, A, B, Bp1, c1, duh, dvh;  // 1/dt, A, B, B + 1, 1/dt + (B + 1), D_u h^-2, D_v h^-2
};

// ((W - c) + (E - c)) + ((S - c) + (N - c)) on the periodic grid: for a smooth state every
// difference of neighbours is exact, so F keeps no rounding floor of order eps * D h^-2 (the form
// Sum - 4c would cancel values near 1 before the multiplication by D h^-2).
__device__ __forceinline__ double lap5(const double* __restrict__ a, int n, int i, int j, double c) {
    const int jm = j == 0 ? n - 1 : j - 1, jp = j + 1 == n ? 0 : j + 1;
    const int im = i == 0 ? n - 1 : i - 1, ip = i + 1 == n ? 0 : i + 1;
    const size_t r = (size_t)i * n;
    return ((a[r + jm] - c) + (a[r + jp] - c)) + ((a[(size_t)im * n + j] - c) + (a[(size_t)ip * n + j] - c));
}

// F(w) = (w - w_prev)/dt - diag(D_u, D_v) h^-2 L w - reaction, as FMA chains (the kernel is bound
// by the FP64 pipe, not by HBM):
//   F_u = fma(B+1, u, fma(-u^2, v, fma(-D_u h^-2, L u, fma(u - u_prev, 1/dt, -A))))
//   F_v = fma(u^2, v, fma(-B, u, fma(-D_v h^-2, L v, (v - v_prev) / dt)));
// optionally ||F||.  L u is lap5's ((W - c) + (E - c)) + ((S - c) + (N - c)), with each neighbour
// difference computed once and shared: a point forms its east difference E - c and takes its west
// one as minus the east difference of the lane to its left (RN(a - b) = -RN(b - a) exactly), and
// forms its north difference N - c, keeping it as the next row's minus-south difference while the
// thread marches down its rows.  Five FP64 instructions for each Laplacian instead of seven, the
// same bits.  A warp covers 31 columns: lane 0 is the halo column whose east difference lane 1 needs.
constexpr int kB2EvalRows = 32;  // rows a thread marches
// FIXED (the mixed path's evaluation): each Laplacian as W + E + S + N - 4c in 64-bit fixed point, rounded
// once (lap5_fixed, common.cuh; more accurate than the sum of rounded differences), on the integer pipe
// instead of five FP64 instructions a species.
template <bool NORM, bool FIXED = false>
__global__ void __launch_bounds__(256) k_b2_eval(const double* __restrict__ w, const double* __restrict__ prev,
                                                 double* __restrict__ out, B2Geom G, RedArgs red, double* norm_out) {
    pdl_wait();
    pdl_trigger();
    const int n = G.n;
    const size_t nn = (size_t)n * n;
    const int lane = threadIdx.x;
    const int jr = (int)blockIdx.x * 31 + lane - 1;  // lane 0: the column left of the warp's 31
    const int j = ((jr % n) + n) % n, jp = j + 1 == n ? 0 : j + 1;  // lanes past the grid wrap (any n)
    const bool owner = lane >= 1 && jr < n;
    const double* wu = w;
    const double* wv = w + nn;
    double acc[1] = {0.0};
    const int i0 = ((int)blockIdx.y * 8 + (int)threadIdx.y) * kB2EvalRows, i1 = min(i0 + kB2EvalRows, n);
    if (i0 < n) {
        const int im0 = i0 == 0 ? n - 1 : i0 - 1;
        double u = wu[(size_t)i0 * n + j], v = wv[(size_t)i0 * n + j];
        double su = 0.0, sv = 0.0;  // S - c of row i0 (FIXED: S itself)
        if (FIXED) {
            su = wu[(size_t)im0 * n + j];
            sv = wv[(size_t)im0 * n + j];
        } else {
            su = wu[(size_t)im0 * n + j] - u;
            sv = wv[(size_t)im0 * n + j] - v;
        }
        for (int i = i0; i < i1; ++i) {
            const size_t r = (size_t)i * n, p = r + j;
            const size_t rn = (size_t)(i + 1 == n ? 0 : i + 1) * n;
            const double un = wu[rn + j], vn = wv[rn + j];
            double lu, lv, nu_ = 0.0, nv_ = 0.0;
            if (FIXED) {
                const double Eu = wu[r + jp], Ev = wv[r + jp];
                const double Wu = __shfl_up_sync(0xffffffffu, u, 1), Wv = __shfl_up_sync(0xffffffffu, v, 1);
                lu = lap5_fixed(u, Wu, Eu, su, un);
                lv = lap5_fixed(v, Wv, Ev, sv, vn);
            } else {
                const double eu = wu[r + jp] - u, ev = wv[r + jp] - v;                  // E - c
                const double wu_ = -__shfl_up_sync(0xffffffffu, eu, 1), wv_ = -__shfl_up_sync(0xffffffffu, ev, 1);  // W - c
                nu_ = un - u;                                                           // N - c
                nv_ = vn - v;
                lu = (wu_ + eu) + (su + nu_);
                lv = (wv_ + ev) + (sv + nv_);
            }
            const double uu = u * u;
            const double fu =
                __fma_rn(G.Bp1, u, __fma_rn(-uu, v, __fma_rn(-G.duh, lu, __fma_rn(u - prev[p], G.invdt, -G.A))));
            const double fv = __fma_rn(uu, v, __fma_rn(-G.B, u, __fma_rn(-G.dvh, lv, (v - prev[nn + p]) * G.invdt)));
            if (owner) {
                out[p] = fu;
                out[nn + p] = fv;
                if (NORM) acc[0] = __fma_rn(fv, fv, __fma_rn(fu, fu, acc[0]));
            }
            if (FIXED) {  // the next row's S
                su = u;
                sv = v;
            } else {      // the next row's S - c
                su = -nu_;
                sv = -nv_;
            }
            u = un;
            v = vn;
        }
    }
    if (NORM) {
        __shared__ double sm[1][32];
        block_sum<1>(acc, sm);
        grid_reduce_finish<1>(acc, red, [norm_out] __device__(const double(&t)[1]) { *norm_out = __dsqrt_rn(t[0]); });
    }
}

dim3 b2_eval_grid(int n) {
    return dim3((unsigned)((n + 30) / 31), (unsigned)((n + 8 * kB2EvalRows - 1) / (8 * kB2EvalRows)));
}

// J d with the point block [[c1 - 2uv, -u^2], [2uv - B, 1/dt + u^2]]:
//   (J d)_u = fma(-u^2, dv, fma(-D_u h^-2, L du, a11 du)),  (J d)_v = fma(a22, dv, fma(a21, du, -D_v h^-2 L dv)).
__global__ void __launch_bounds__(256) k_b2_jvp(const double* __restrict__ w, const double* __restrict__ d,
                                                double* __restrict__ out, B2Geom G) {
    pdl_wait();
    pdl_trigger();
    const int n = G.n;
    const size_t nn = (size_t)n * n;
    const int j = blockIdx.x * 32 + threadIdx.x;
    if (j >= n) return;
    for (int i = blockIdx.y * 8 + threadIdx.y; i < n; i += gridDim.y * 8) {
        const size_t p = (size_t)i * n + j;
        const double u = w[p], v = w[nn + p], du = d[p], dv = d[nn + p];
        const double lu = lap5(d, n, i, j, du), lv = lap5(d + nn, n, i, j, dv);
        const double u2 = 2.0 * u, uu = u * u;
        const double a11 = __fma_rn(-u2, v, G.c1), a21 = __fma_rn(u2, v, -G.B), a22 = G.invdt + uu;
        out[p] = __fma_rn(-uu, dv, __fma_rn(-G.duh, lu, a11 * du));
        out[nn + p] = __fma_rn(a22, dv, __fma_rn(a21, du, -G.dvh * lv));
    }
}

// The FP32 Jacobian product's coefficients at the iterate: (2uv, u^2) per point, in FP32 arithmetic.
__global__ void __launch_bounds__(256) k_b2_coef32(const double* __restrict__ w, size_t nn, float2* __restrict__ c) {
    pdl_wait();
    pdl_trigger();
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nn) return;
    const float u = f64_to_f32(w[p]), v = f64_to_f32(w[nn + p]);  // FP32 from the rounded state
    c[p] = make_float2((2.0f * u) * v, u * u);
}

struct B2Geom32 {
    int n;
    float invdt, B, c1, duh, dvh;
};

__device__ __forceinline__ float to_f32(double x) { return f64_to_f32(x); }
__device__ __forceinline__ float to_f32(float x) { return x; }

// J d in FP32 arithmetic (FP64 out; d in FP64 or already in FP32): a 32 x 8 tile of both components
// with its one-point periodic halo is rounded to FP32 once per point (integer-pipe conversion) into
// shared memory.
template <class VT>
__global__ void __launch_bounds__(256) k_b2_jvp32(const float2* __restrict__ coef, const VT* __restrict__ d,
                                                  double* __restrict__ out, B2Geom32 G) {
    pdl_wait();
    pdl_trigger();
    constexpr int TX = 32, TY = 8;
    __shared__ float tu[TY + 2][TX + 3], tv[TY + 2][TX + 3];
    const int n = G.n;
    const size_t nn = (size_t)n * n;
    const int i0 = blockIdx.y * TY, j0 = blockIdx.x * TX;
    const int tid = threadIdx.y * TX + threadIdx.x;
    for (int idx = tid; idx < (TY + 2) * (TX + 2); idx += TX * TY) {
        const int a = idx / (TX + 2), b = idx - a * (TX + 2);
        const int gi = (i0 - 1 + a + n) % n, gj = (j0 - 1 + b + n) % n;
        const size_t q = (size_t)gi * n + gj;
        tu[a][b] = to_f32(d[q]);
        tv[a][b] = to_f32(d[nn + q]);
    }
    __syncthreads();
    const int i = i0 + threadIdx.y, j = j0 + threadIdx.x;
    if (i >= n || j >= n) return;
    const int a = threadIdx.y + 1, b = threadIdx.x + 1;
    const float du = tu[a][b], dv = tv[a][b];
    const float lu = ((tu[a][b - 1] - du) + (tu[a][b + 1] - du)) + ((tu[a - 1][b] - du) + (tu[a + 1][b] - du));
    const float lv = ((tv[a][b - 1] - dv) + (tv[a][b + 1] - dv)) + ((tv[a - 1][b] - dv) + (tv[a + 1][b] - dv));
    const size_t p = (size_t)i * n + j;
    const float2 c = coef[p];
    const float a11 = G.c1 - c.x, a21 = c.x - G.B, a22 = G.invdt + c.y;
    const float ou = __fmaf_rn(-c.y, dv, __fmaf_rn(-G.duh, lu, a11 * du));
    const float ov = __fmaf_rn(a22, dv, __fmaf_rn(a21, du, -G.dvh * lv));
    out[p] = f32_to_f64(ou);
    out[nn + p] = f32_to_f64(ov);
}

dim3 b2_grid(int n) {
    const unsigned gx = (unsigned)((n + 31) / 32);
    const unsigned rows = (unsigned)((n + 7) / 8);
    const unsigned gy = std::max(1u, std::min(rows, (unsigned)kMaxRedBlocks / gx));
    return dim3(gx, gy);
}

// The same product from an FP32 d (the multigrid's output): no conversion, so no shared-memory
// tile — neighbours come through L1; the arithmetic is k_b2_jvp32's, operation for operation.  OT =
// float stores the FP32 result as it is, OT = double widens it.
template <class OT>
__global__ void __launch_bounds__(256) k_b2_jvp32f(const float2* __restrict__ coef, const float* __restrict__ d,
                                                   OT* __restrict__ out, B2Geom32 G) {
    pdl_wait();
    pdl_trigger();
    const int n = G.n;
    const size_t nn = (size_t)n * n;
    const int j = blockIdx.x * 32 + threadIdx.x;
    if (j >= n) return;
    const int jm = j == 0 ? n - 1 : j - 1, jp = j + 1 == n ? 0 : j + 1;
    for (int i = blockIdx.y * 8 + threadIdx.y; i < n; i += gridDim.y * 8) {
        const int im = i == 0 ? n - 1 : i - 1, ip = i + 1 == n ? 0 : i + 1;
        const size_t r = (size_t)i * n, p = r + j;
        const float du = d[p], dv = d[nn + p];
        const float lu = ((d[r + jm] - du) + (d[r + jp] - du)) + ((d[(size_t)im * n + j] - du) + (d[(size_t)ip * n + j] - du));
        const float* e = d + nn;
        const float lv = ((e[r + jm] - dv) + (e[r + jp] - dv)) + ((e[(size_t)im * n + j] - dv) + (e[(size_t)ip * n + j] - dv));
        const float2 c = coef[p];
        const float a11 = G.c1 - c.x, a21 = c.x - G.B, a22 = G.invdt + c.y;
        const float ru = __fmaf_rn(-c.y, dv, __fmaf_rn(-G.duh, lu, a11 * du));
        const float rv = __fmaf_rn(a22, dv, __fmaf_rn(a21, du, -G.dvh * lv));
        if constexpr (sizeof(OT) == 4) {
            out[p] = ru;
            out[nn + p] = rv;
        } else {
            out[p] = f32_to_f64(ru);
            out[nn + p] = f32_to_f64(rv);
        }
    }
}

// ============================================================================== BrussMG2D kernels
template <class T> struct P2;
template <> struct P2<float> { using t = float2; };
template <> struct P2<double> { using t = double2; };

template <class T>
struct Blk {
    T k11, k12, k21, k22;
};

__device__ __forceinline__ Blk<float> load_blk(const float* __restrict__ K, size_t p) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(K) + p);
    return {q.x, q.y, q.z, q.w};
}
__device__ __forceinline__ Blk<double> load_blk(const double* __restrict__ K, size_t p) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(K) + 2 * p);
    const double2 b = __ldg(reinterpret_cast<const double2*>(K) + 2 * p + 1);
    return {a.x, a.y, b.x, b.y};
}
// the same from shared memory (no read-only-cache path)
__device__ __forceinline__ Blk<float> load_blk_s(const float* K, size_t p) {
    const float4 q = reinterpret_cast<const float4*>(K)[p];
    return {q.x, q.y, q.z, q.w};
}
__device__ __forceinline__ Blk<double> load_blk_s(const double* K, size_t p) {
    const double2 a = reinterpret_cast<const double2*>(K)[2 * p];
    const double2 b = reinterpret_cast<const double2*>(K)[2 * p + 1];
    return {a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void store_blk(float* K, size_t p, const Blk<float>& k) {
    reinterpret_cast<float4*>(K)[p] = make_float4(k.k11, k.k12, k.k21, k.k22);
}
__device__ __forceinline__ void store_blk(double* K, size_t p, const Blk<double>& k) {
    reinterpret_cast<double2*>(K)[2 * p] = make_double2(k.k11, k.k12);
    reinterpret_cast<double2*>(K)[2 * p + 1] = make_double2(k.k21, k.k22);
}

template <class T>
__device__ __forceinline__ typename P2<T>::t ld2(const T* a, size_t p) {
    return reinterpret_cast<const typename P2<T>::t*>(a)[p];
}
template <class T>
__device__ __forceinline__ void st2(T* a, size_t p, T u, T v) {
    typename P2<T>::t q;
    q.x = u;
    q.y = v;
    reinterpret_cast<typename P2<T>::t*>(a)[p] = q;
}

// Point-block Gauss-Seidel update: (K + 4 diag(s_u, s_v)) (u, v) = (b_u + s_u S_u, b_v + s_v S_v),
// S = ((W + E) + S) + N, by Cramer's rule with two divisions.
template <class T>
__device__ __forceinline__ void block_update(const Blk<T>& k, T su, T sv, T su4, T sv4, T bu, T bv, T Su, T Sv,
                                             T& u, T& v) {
    const T ru = bu + su * Su;
    const T rv = bv + sv * Sv;
    const T m11 = k.k11 + su4, m22 = k.k22 + sv4;
    const T det = m11 * m22 - k.k12 * k.k21;
    u = (m22 * ru - k.k12 * rv) / det;
    v = (m11 * rv - k.k21 * ru) / det;
}

// One level's constants in the multigrid's precision, formed on the host: a kernel converting
// doubles per thread would spend GB300's narrow FP64 pipe on it (a few FP64 instructions per
// thread bound a one-point-per-thread FP32 pass).
template <class T>
struct LvlArgs {
    int n;
    T su, sv, su4, sv4;  // s_u = D_u h^-2, s_v, 4 s_u, 4 s_v
};

// FP64 <-> T without the FP64 pipe for T = float (integer-path conversions, same rounding).
template <class T> __device__ __forceinline__ T from_f64(double x);
template <> __device__ __forceinline__ float from_f64<float>(double x) { return f64_to_f32(x); }
template <> __device__ __forceinline__ double from_f64<double>(double x) { return x; }
// a right-hand side read as FP64 or as FP32 into the level type
template <class T> __device__ __forceinline__ T from_in(double x) { return from_f64<T>(x); }
template <class T> __device__ __forceinline__ T from_in(float x) {
    if constexpr (sizeof(T) == 4) return x;
    else return f32_to_f64(x);
}
__device__ __forceinline__ double to_f64(float x) { return f32_to_f64(x); }
__device__ __forceinline__ double to_f64(double x) { return x; }

// Storage index of point (i, j) of an n x n level (n even): colour-split, each colour's points in
// row-major order, colour (i + j) & 1 first-half / second-half — a colour pass then reads and
// writes only whole cache lines of the colours it touches.  The four neighbours of a point are all
// of the other colour, in its rows i and i +- 1 at column index j/2 or j/2 +- 1.
__device__ __forceinline__ size_t pidx(int n, int i, int j) {
    const int half = n >> 1;
    return (size_t)((i + j) & 1) * ((size_t)n * half) + (size_t)i * half + (j >> 1);
}

template <class T>
__device__ __forceinline__ void nbr_sums(const T* __restrict__ X, int n, int i, int j, T& Su, T& Sv) {
    const int jm = j == 0 ? n - 1 : j - 1, jp = j + 1 == n ? 0 : j + 1;
    const int im = i == 0 ? n - 1 : i - 1, ip = i + 1 == n ? 0 : i + 1;
    const auto w = ld2(X, pidx(n, i, jm)), e = ld2(X, pidx(n, i, jp)), s = ld2(X, pidx(n, im, j)),
               nn = ld2(X, pidx(n, ip, j));
    Su = ((w.x + e.x) + s.x) + nn.x;
    Sv = ((w.y + e.y) + s.y) + nn.y;
}

enum { kBPassNormal = 0, kBPassFirst = 1, kBPassLast = 2 };

// One colour of red-black point-block Gauss-Seidel on one level.  Thread (jj, i) owns the pair
// of row i's points 2jj and 2jj + 1 (one of each colour) and updates the one of this colour; a warp
// covers 32 consecutive points of one colour.
//  Normal: x_c updated from the other colour.
//  First (colour 0, x = 0 before the pass): x_0 = block^-1 b (neighbour sums are zeros), x_1 = 0;
//    on the finest level the right-hand side is read from r (FP64 planes) and stored as b.
//  Last (finest level, colour 0, the cycle's final pass): also writes z (FP64 planes) for both points,
//    or, for an FP32 consumer, the same values as FP32 planes z32.
template <class T, int MODE, class RT = double>
__global__ void __launch_bounds__(256) k_bmg_pass(T* __restrict__ X, T* __restrict__ Bv, const T* __restrict__ K,
                                                  LvlArgs<T> L, int colour, const RT* __restrict__ r64,
                                                  double* __restrict__ z64, float* __restrict__ z32 = nullptr) {
    pdl_wait();
    pdl_trigger();
    const int n = L.n;
    const int jj = blockIdx.x * 32 + threadIdx.x;
    const int i = blockIdx.y * 8 + threadIdx.y;
    if (i >= n || 2 * jj >= n) return;
    const T su = L.su, sv = L.sv, su4 = L.su4, sv4 = L.sv4;
    const int j = 2 * jj + ((i + colour) & 1);
    const int jo = 2 * jj + 1 - ((i + colour) & 1);
    const size_t p = pidx(n, i, j), po = pidx(n, i, jo);                // level storage
    const size_t pn = (size_t)i * n + j, pon = (size_t)i * n + jo;      // r and z: natural planes
    const size_t nn = (size_t)n * n;
    T bu, bv;
    if (MODE == kBPassFirst && r64) {
        bu = from_in<T>(r64[pn]);
        bv = from_in<T>(r64[nn + pn]);
        st2(Bv, p, bu, bv);
        st2(Bv, po, from_in<T>(r64[pon]), from_in<T>(r64[nn + pon]));
    } else {
        const auto b = ld2(Bv, p);
        bu = b.x;
        bv = b.y;
    }
    T Su, Sv;
    if (MODE == kBPassFirst) {
        Su = T(0);
        Sv = T(0);
    } else {
        nbr_sums(X, n, i, j, Su, Sv);
    }
    T u, v;
    block_update(load_blk(K, p), su, sv, su4, sv4, bu, bv, Su, Sv, u, v);
    st2(X, p, u, v);
    if (MODE == kBPassFirst) st2(X, po, T(0), T(0));
    if (MODE == kBPassLast) {
        const auto o = ld2(X, po);
        if (z64) {
            z64[pn] = to_f64(u);
            z64[nn + pn] = to_f64(v);
            z64[pon] = to_f64(o.x);
            z64[nn + pon] = to_f64(o.y);
        }
        if constexpr (sizeof(T) == 4) {
            if (z32) {  // or the values unwidened, for an FP32 consumer
                z32[pn] = u;
                z32[nn + pn] = v;
                z32[pon] = o.x;
                z32[nn + pon] = o.y;
            }
        }
    }
}

// Residual r = b - (K x - diag(s) (S - 4x)) of one level at point (i, j).
template <class T, bool SMEM_K = false>
__device__ __forceinline__ void resid_at(const T* X, const T* Bv, const T* K, int n, int i, int j, T su, T sv, T& ru,
                                         T& rv) {
    const size_t p = pidx(n, i, j);
    const auto x = ld2(X, p);
    const auto bb = ld2(Bv, p);
    const Blk<T> k = SMEM_K ? load_blk_s(K, p) : load_blk(K, p);
    T Su, Sv;
    nbr_sums(X, n, i, j, Su, Sv);
    ru = bb.x - ((k.k11 * x.x + k.k12 * x.y) + su * (T(4) * x.x - Su));
    rv = bb.y - ((k.k21 * x.x + k.k22 * x.y) + sv * (T(4) * x.y - Sv));
}

// 9-point full weighting ((4c + 2((W + E) + (S + N))) + (((SW + SE) + NW) + NE)) / 16; S is row i-1.
template <class T>
__device__ __forceinline__ T fw9(T c, T w, T e, T s, T n, T sw, T se, T nw, T ne) {
    const T edge = (w + e) + (s + n);
    const T corner = ((sw + se) + nw) + ne;
    return ((T(4) * c + T(2) * edge) + corner) * T(0.0625);
}

// Residual of the finest-level points that a 16 x 16 tile of coarse points covers (33 x 33,
// periodic), kept in shared memory, then full weighting into the coarse right-hand side.
template <class T>
__global__ void __launch_bounds__(256) k_bmg_restrict(const T* __restrict__ X, const T* __restrict__ Bv,
                                                      const T* __restrict__ K, LvlArgs<T> L, T* __restrict__ Bc) {
    pdl_wait();
    pdl_trigger();
    constexpr int TS = 16, FS = 2 * TS + 1;
    __shared__ T su_s[FS][FS + 1], sv_s[FS][FS + 1];
    const int nf = L.n, nc = nf / 2;
    const int I0 = blockIdx.y * TS, J0 = blockIdx.x * TS;
    const int tid = threadIdx.y * TS + threadIdx.x;
    const T su = L.su, sv = L.sv;
    for (int idx = tid; idx < FS * FS; idx += TS * TS) {
        const int a = idx / FS, b = idx - a * FS;
        const int fi = (2 * I0 - 1 + a + nf) % nf, fj = (2 * J0 - 1 + b + nf) % nf;
        resid_at(X, Bv, K, nf, fi, fj, su, sv, su_s[a][b], sv_s[a][b]);
    }
    __syncthreads();
    const int I = I0 + threadIdx.y, J = J0 + threadIdx.x;
    if (I >= nc || J >= nc) return;
    const int a = 2 * threadIdx.y + 1, b = 2 * threadIdx.x + 1;
    auto fw = [a, b](const T (*f)[FS + 1]) {
        return fw9(f[a][b], f[a][b - 1], f[a][b + 1], f[a - 1][b], f[a + 1][b], f[a - 1][b - 1], f[a - 1][b + 1],
                   f[a + 1][b - 1], f[a + 1][b + 1]);
    };
    st2(Bc, pidx(nc, I, J), fw(su_s), fw(sv_s));
}

// x_fine += bilinear periodic interpolation of x_coarse at the fine points (2I + {0,1}, 2J + {0,1}).
template <class T>
__device__ __forceinline__ void prolong_point(const T* Xc, int nc, int I, int J, T* Xf) {
    const int I1 = I + 1 == nc ? 0 : I + 1, J1 = J + 1 == nc ? 0 : J + 1;
    const auto c00 = ld2(Xc, pidx(nc, I, J)), c10 = ld2(Xc, pidx(nc, I1, J));
    const auto c01 = ld2(Xc, pidx(nc, I, J1)), c11 = ld2(Xc, pidx(nc, I1, J1));
    const int nf = 2 * nc;
    const size_t f00 = pidx(nf, 2 * I, 2 * J), f10 = pidx(nf, 2 * I + 1, 2 * J);
    const size_t f01 = pidx(nf, 2 * I, 2 * J + 1), f11 = pidx(nf, 2 * I + 1, 2 * J + 1);
    // the four fine pairs are loaded before any is stored (the compiler cannot tell the addresses apart)
    const auto x00 = ld2(Xf, f00), x10 = ld2(Xf, f10), x01 = ld2(Xf, f01), x11 = ld2(Xf, f11);
    st2(Xf, f00, x00.x + c00.x, x00.y + c00.y);
    st2(Xf, f10, x10.x + T(0.5) * (c00.x + c10.x), x10.y + T(0.5) * (c00.y + c10.y));
    st2(Xf, f01, x01.x + T(0.5) * (c00.x + c01.x), x01.y + T(0.5) * (c00.y + c01.y));
    st2(Xf, f11, x11.x + T(0.25) * (((c00.x + c10.x) + c01.x) + c11.x),
        x11.y + T(0.25) * (((c00.y + c10.y) + c01.y) + c11.y));
}

template <class T>
__global__ void __launch_bounds__(256) k_bmg_prolong(const T* __restrict__ Xc, int nc, T* __restrict__ Xf) {
    pdl_wait();
    pdl_trigger();
    const int J = blockIdx.x * 32 + threadIdx.x;
    const int I = blockIdx.y * 8 + threadIdx.y;
    if (I >= nc || J >= nc) return;
    prolong_point(Xc, nc, I, J, Xf);
}

// The coarsest level in one block: x = 0, then `sweeps` red-black sweeps (colour 0, 1).
template <class T>
__global__ void __launch_bounds__(1024) k_bmg_coarsest(T* __restrict__ X, const T* __restrict__ Bv,
                                                       const T* __restrict__ K, LvlArgs<T> L, int sweeps) {
    pdl_wait();
    pdl_trigger();
    const int n = L.n;
    const int nn = n * n;
    const T su = L.su, sv = L.sv, su4 = L.su4, sv4 = L.sv4;
    for (int p = threadIdx.x; p < nn; p += blockDim.x) st2(X, p, T(0), T(0));
    __syncthreads();
    for (int s = 0; s < sweeps; ++s) {
        for (int c = 0; c < 2; ++c) {
            for (int p = threadIdx.x; p < nn; p += blockDim.x) {
                const int i = p / n, j = p - i * n;
                if (((i + j) & 1) != c) continue;
                const size_t q = pidx(n, i, j);
                T Su, Sv, u, v;
                nbr_sums(X, n, i, j, Su, Sv);
                const auto b = ld2(Bv, q);
                block_update(load_blk(K, q), su, sv, su4, sv4, b.x, b.y, Su, Sv, u, v);
                st2(X, q, u, v);
            }
            __syncthreads();
        }
    }
}

// The small levels below the finest (n <= 64 in FP32, n <= 32 in FP64) as one block: every tail
// level's pairs x, b and blocks K live in shared memory (8 n^2 values a level, at most 175 KB), and
// the block runs their whole V-cycle — the same per-point arithmetic as the level kernels, so the
// result is the same to the bit.  desc[k] describes tail level k (k = 0 the finest of them): its
// n, the offset of its x in the shared buffer (b follows at offset + 2 n^2, K at offset + 4 n^2),
// s_u, s_v and its blocks in global memory (copied in at the start).
struct TailLvl {
    int n, off;
    const void* K;
    LvlArgs<double> d;  // the level's constants in FP64 and in FP32 (formed on the host: one SM's
    LvlArgs<float> f;   // FP64 pipe would take tens of microseconds to convert them per pass)
};
template <class T> __device__ __forceinline__ const LvlArgs<T>& tail_args(const TailLvl& L);
template <> __device__ __forceinline__ const LvlArgs<double>& tail_args<double>(const TailLvl& L) { return L.d; }
template <> __device__ __forceinline__ const LvlArgs<float>& tail_args<float>(const TailLvl& L) { return L.f; }

// threads of the one-CTA tail: 1024 in FP32 (64 registers, no spills), 512 in FP64 (which would spill at 1024)
template <class T>
constexpr int kBmgTailThreads = sizeof(T) == 4 ? 1024 : 512;
template <class T>
__global__ void __launch_bounds__(kBmgTailThreads<T>, 1) k_bmg_tail(const TailLvl* __restrict__ desc, int count, int pre, int post,
                                                     int sweeps, const T* __restrict__ Bin, T* __restrict__ Xout) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ __align__(16) unsigned char bmg_smem[];
    T* base = reinterpret_cast<T*>(bmg_smem);
    // Levels with n <= 8 (at most 32 points of a colour) are run by warp 0 alone, separated by
    // __syncwarp instead of block barriers; `kw` is the first of them (count if none).
    int kw = count;
    for (int k = 0; k < count; ++k)
        if (desc[k].n <= 8) {
            kw = k;
            break;
        }
    const bool warp0 = threadIdx.x < 32;
    // one colour pass of level k by threads [0, nt); then the barrier of that group
    auto pass = [&](int k, int colour, bool first) {
        const bool small = k >= kw;
        const int tid = threadIdx.x, nt = small ? 32 : blockDim.x;
        const TailLvl L = desc[k];
        const int n = L.n, half = n / 2;
        T* X = base + L.off;
        const T* Bv = X + 2 * n * n;
        const T* K = X + 4 * n * n;
        const LvlArgs<T>& A = tail_args<T>(L);
        const T su = A.su, sv = A.sv, su4 = A.su4, sv4 = A.sv4;
        for (int idx = tid; idx < n * half; idx += nt) {
            const int i = idx / half, jj = idx - i * half;
            const int j = 2 * jj + ((i + colour) & 1), jo = 2 * jj + 1 - ((i + colour) & 1);
            const size_t p = pidx(n, i, j);
            const auto b = ld2(Bv, p);
            T Su = T(0), Sv = T(0), u, v;
            if (!first) nbr_sums(X, n, i, j, Su, Sv);
            block_update(load_blk_s(K, p), su, sv, su4, sv4, b.x, b.y, Su, Sv, u, v);
            st2(X, p, u, v);
            if (first) st2(X, pidx(n, i, jo), T(0), T(0));
        }
        if (small) __syncwarp();
        else __syncthreads();
    };
    // residual of level k, full-weighted into the right-hand side of level k + 1
    auto restrict_to = [&](int k) {
        const bool small = k + 1 >= kw && k >= kw;
        const int tid = threadIdx.x, nt = small ? 32 : blockDim.x;
        const TailLvl L = desc[k], C = desc[k + 1];
        const int nf = L.n, nc = C.n;
        const T* X = base + L.off;
        const T* Bv = X + 2 * nf * nf;
        const T* K = X + 4 * nf * nf;
        T* Bc = base + C.off + 2 * nc * nc;
        const T su = tail_args<T>(L).su, sv = tail_args<T>(L).sv;
        for (int idx = tid; idx < nc * nc; idx += nt) {
            const int I = idx / nc, J = idx - I * nc;
            const int i = 2 * I, j = 2 * J;
            const int im = i == 0 ? nf - 1 : i - 1, ip = i + 1, jm = j == 0 ? nf - 1 : j - 1, jp = j + 1;
            // fw9's sums in its order, accumulated as the residuals are formed (fewer live registers)
            T cu, cv, au, av, bu, bv;
            resid_at<T, true>(X, Bv, K, nf, i, j, su, sv, cu, cv);
            resid_at<T, true>(X, Bv, K, nf, i, jm, su, sv, au, av);
            resid_at<T, true>(X, Bv, K, nf, i, jp, su, sv, bu, bv);
            const T weu = au + bu, wev = av + bv;
            resid_at<T, true>(X, Bv, K, nf, im, j, su, sv, au, av);
            resid_at<T, true>(X, Bv, K, nf, ip, j, su, sv, bu, bv);
            const T edgeu = weu + (au + bu), edgev = wev + (av + bv);
            resid_at<T, true>(X, Bv, K, nf, im, jm, su, sv, au, av);
            resid_at<T, true>(X, Bv, K, nf, im, jp, su, sv, bu, bv);
            T coru = au + bu, corv = av + bv;
            resid_at<T, true>(X, Bv, K, nf, ip, jm, su, sv, au, av);
            coru = coru + au;
            corv = corv + av;
            resid_at<T, true>(X, Bv, K, nf, ip, jp, su, sv, au, av);
            coru = coru + au;
            corv = corv + av;
            st2(Bc, pidx(nc, I, J), ((T(4) * cu + T(2) * edgeu) + coru) * T(0.0625),
                ((T(4) * cv + T(2) * edgev) + corv) * T(0.0625));
        }
        if (small) __syncwarp();
        else __syncthreads();
    };
    auto prolong_from = [&](int k) {  // level k + 1 into level k
        const bool small = k >= kw;
        const int tid = threadIdx.x, nt = small ? 32 : blockDim.x;
        const int nc = desc[k + 1].n;
        const T* Xc = base + desc[k + 1].off;
        T* Xf = base + desc[k].off;
        for (int idx = tid; idx < nc * nc; idx += nt) prolong_point(Xc, nc, idx / nc, idx % nc, Xf);
        if (small) __syncwarp();
        else __syncthreads();
    };
    auto down = [&](int k) {
        pass(k, 0, true);
        pass(k, 1, false);
        for (int s = 1; s < pre; ++s) {
            pass(k, 0, false);
            pass(k, 1, false);
        }
        restrict_to(k);
    };
    auto up = [&](int k) {
        prolong_from(k);
        for (int s = 0; s < post; ++s) {
            pass(k, 1, false);
            pass(k, 0, false);
        }
    };
    auto coarsest = [&]() {
        const int kc = count - 1, n = desc[kc].n;
        const bool small = kc >= kw;
        const int tid = threadIdx.x, nt = small ? 32 : blockDim.x;
        T* X = base + desc[kc].off;
        for (int q = tid; q < 2 * n * n; q += nt) X[q] = T(0);
        if (small) __syncwarp();
        else __syncthreads();
        for (int s = 0; s < sweeps; ++s) {
            pass(kc, 0, false);
            pass(kc, 1, false);
        }
    };
    {
        const int n0 = desc[0].n;
        T* B0 = base + desc[0].off + 2 * n0 * n0;
        for (int q = threadIdx.x; q < 2 * n0 * n0; q += blockDim.x) B0[q] = Bin[q];
        for (int k = 0; k < count; ++k) {
            const int nk = desc[k].n;
            const float4* src = static_cast<const float4*>(desc[k].K);
            float4* dst = reinterpret_cast<float4*>(base + desc[k].off + 4 * nk * nk);
            const int n16 = (int)(4 * (size_t)nk * nk * sizeof(T) / 16);
            for (int q = threadIdx.x; q < n16; q += blockDim.x) dst[q] = __ldg(src + q);
        }
    }
    __syncthreads();
    // block-wide levels down to kw (restricting into kw last)
    for (int k = 0; k + 1 < count && k < kw; ++k) down(k);
    if (kw < count) {
        // the warp-sized levels: the rest of the V-cycle from level kw down and back up, warp 0 only
        if (warp0) {
            for (int k = kw; k + 1 < count; ++k) down(k);
            coarsest();
            for (int k = count - 2; k >= kw; --k) up(k);
        }
        __syncthreads();
    } else {
        coarsest();
    }
    for (int k = (kw < count - 1 ? kw : count - 1) - 1; k >= 0; --k) up(k);
    const int n0 = desc[0].n;
    const T* X0 = base + desc[0].off;
    for (int q = threadIdx.x; q < 2 * n0 * n0; q += blockDim.x) Xout[q] = X0[q];
}

// K at the finest level from the FP64 state: [[1/dt + B + 1 - 2uv, -u^2], [2uv - B, 1/dt + u^2]];
// in FP64 for the FP64 multigrid, in FP32 from the rounded state for the FP32 one (a preconditioner
// needs no more, and FP64 arithmetic would bound the kernel).
__device__ __forceinline__ void kfine_point(double u, double v, double c1, double c2, double B, Blk<double>& k) {
    k.k11 = c1 - (2.0 * u) * v;
    k.k12 = -(u * u);
    k.k21 = (2.0 * u) * v - B;
    k.k22 = c2 + u * u;
}
__device__ __forceinline__ void kfine_point(double u, double v, float c1, float c2, float B, Blk<float>& k) {
    const float u32 = f64_to_f32(u), v32 = f64_to_f32(v);
    const float uv2 = (2.0f * u32) * v32, uu = u32 * u32;
    k.k11 = c1 - uv2;
    k.k12 = -uu;
    k.k21 = uv2 - B;
    k.k22 = c2 + uu;
}

// c1 = 1/dt + (B + 1), c2 = 1/dt and B in the multigrid's precision (rounded on the host)
template <class T>
__global__ void __launch_bounds__(256) k_bmg_kfine(const double* __restrict__ w, int n, T c1, T c2, T B,
                                                   T* __restrict__ K) {
    pdl_wait();
    pdl_trigger();
    const size_t nn = (size_t)n * n;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nn) return;
    const int i = (int)(p / n), j = (int)(p - (size_t)i * n);
    Blk<T> k;
    kfine_point(w[p], w[nn + p], c1, c2, B, k);
    store_blk(K, pidx(n, i, j), k);
}

// Full weighting of the four block components to the next coarser level.
template <class T>
__global__ void __launch_bounds__(256) k_bmg_krestrict(const T* __restrict__ Kf, int nf, T* __restrict__ Kc) {
    pdl_wait();
    pdl_trigger();
    const int nc = nf / 2;
    const int J = blockIdx.x * 32 + threadIdx.x;
    const int I = blockIdx.y * 8 + threadIdx.y;
    if (I >= nc || J >= nc) return;
    const int i = 2 * I, j = 2 * J;
    const int im = i == 0 ? nf - 1 : i - 1, ip = i + 1, jm = j == 0 ? nf - 1 : j - 1, jp = j + 1;
    auto at = [Kf, nf](int a, int b) { return load_blk(Kf, pidx(nf, a, b)); };
    const Blk<T> c = at(i, j), w = at(i, jm), e = at(i, jp), s = at(im, j), nth = at(ip, j);
    const Blk<T> sw = at(im, jm), se = at(im, jp), nw = at(ip, jm), ne = at(ip, jp);
    auto fw = [](T ctr, T w_, T e_, T s_, T n_, T sw_, T se_, T nw_, T ne_) {
        const T edge = (w_ + e_) + (s_ + n_);
        const T corner = ((sw_ + se_) + nw_) + ne_;
        return ((T(4) * ctr + T(2) * edge) + corner) * T(0.0625);
    };
    Blk<T> o;
    o.k11 = fw(c.k11, w.k11, e.k11, s.k11, nth.k11, sw.k11, se.k11, nw.k11, ne.k11);
    o.k12 = fw(c.k12, w.k12, e.k12, s.k12, nth.k12, sw.k12, se.k12, nw.k12, ne.k12);
    o.k21 = fw(c.k21, w.k21, e.k21, s.k21, nth.k21, sw.k21, se.k21, nw.k21, ne.k21);
    o.k22 = fw(c.k22, w.k22, e.k22, s.k22, nth.k22, sw.k22, se.k22, nw.k22, ne.k22);
    store_blk(Kc, pidx(nc, I, J), o);
}

// FP64 planes <-> interleaved level pairs (used only when the finest level is also the coarsest).
template <class T, class RT = double>
__global__ void k_bmg_in(const RT* __restrict__ r, int n, T* __restrict__ B) {
    pdl_wait();
    pdl_trigger();
    const size_t nn = (size_t)n * n;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nn) return;
    const int i = (int)(p / n), j = (int)(p - (size_t)i * n);
    st2(B, pidx(n, i, j), from_in<T>(r[p]), from_in<T>(r[nn + p]));
}
template <class T>
__global__ void k_bmg_out(const T* __restrict__ X, int n, double* __restrict__ z) {
    pdl_wait();
    pdl_trigger();
    const size_t nn = (size_t)n * n;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nn) return;
    const int i = (int)(p / n), j = (int)(p - (size_t)i * n);
    const auto x = ld2(X, pidx(n, i, j));
    z[p] = to_f64(x.x);
    z[nn + p] = to_f64(x.y);
}

constexpr int kBmgCoarsestSweeps = 30;
constexpr int kBmgOneBlockPoints = 4096;
constexpr int kBmgTailMaxN = 64;  // levels this small (below the finest; half in FP64) run in the one-block tail

}  // namespace

// ============================================================================== Brusselator1D
Brusselator1D::Brusselator1D(Context& ctx, size_t n, double dt) : NonlinearOp(ctx), n_(n), dt_(dt) {
    if (n == 0 || !(dt > 0.0) || !std::isfinite(dt))
        throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "Brusselator1DStep requires valid n and dt");
    if (n > (size_t)1 << 28) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "Brusselator1DStep grid too large");
    h_ = 1.0 / (static_cast<double>(n) + 1.0);
    h2inv_ = 1.0 / (h_ * h_);
    // previous state u = 1 + sin(2 pi x), v = 3 at x = (i + 1) h (brusselator1d.hpp:30-37)
    std::vector<double> prev(2 * n);
    const double pi = std::acos(-1.0);
    for (size_t i = 0; i < n; ++i) {
        const double x = (static_cast<double>(i) + 1.0) * h_;
        prev[i] = 1.0 + std::sin(2.0 * pi * x);
        prev[n + i] = 3.0;
    }
    prev_.resize(2 * n);
    NUMA_CUDA(cudaMemcpyAsync(prev_.p, prev.data(), 2 * n * sizeof(double), cudaMemcpyHostToDevice, ctx_.stream));
    ctx_.sync();
}

static B1Geom b1_geom(size_t n, double dt, double h2inv) {
    B1Geom G;
    G.n = (int)n;
    G.invdt = 1.0 / dt;
    G.h2inv = h2inv;
    G.alpha = Brusselator1D::kAlpha;
    G.A = Brusselator1D::kA;
    G.B = Brusselator1D::kB;
    G.base = 1.0 / dt + 2.0 * Brusselator1D::kAlpha * h2inv;
    return G;
}

void Brusselator1D::eval(const double* x, double* out, double*, double* norm_out) {
    launch_pdl(k_b1_eval, (unsigned)((n_ + 255) / 256), 256, 0, ctx_.stream, x, prev_.p, out, b1_geom(n_, dt_, h2inv_));
    ctx_.count_launch();
    ctx_.check_launch("Brusselator1D eval");
    if (norm_out) dev_norm2(ctx_, out, size(), norm_out);
}

void Brusselator1D::jvp_at(const double* x, const double* v, double* out) {
    launch_pdl(k_b1_jvp, (unsigned)((n_ + 255) / 256), 256, 0, ctx_.stream, x, v, out, b1_geom(n_, dt_, h2inv_));
    ctx_.count_launch();
    ctx_.check_launch("Brusselator1D jvp");
}

void Brusselator1D::d2(const double* x, const double*, const double* v, double* out) {
    launch_pdl(k_bruss_d2, (unsigned)((n_ + 255) / 256), 256, 0, ctx_.stream, x, v, out, n_);
    ctx_.count_launch();
    ctx_.check_launch("Brusselator1D d2");
}

void Brusselator1D::blocks(const double* x, double* a) {
    launch_pdl(k_b1_blocks, (unsigned)((n_ + 255) / 256), 256, 0, ctx_.stream, x, a, b1_geom(n_, dt_, h2inv_));
    ctx_.count_launch();
    ctx_.check_launch("Brusselator1D blocks");
}

void brusselator_block_apply(Context& ctx, const double* a, const double* r, double* z, size_t n) {
    launch_pdl(k_b1_block_apply, (unsigned)((n + 255) / 256), 256, 0, ctx.stream, a, r, z, (int)n);
    ctx.count_launch();
    ctx.check_launch("BrusselatorJacobi apply");
}

namespace {
// BrusselatorJacobi (brusselator1d.hpp:194-222): make(x) forms the point blocks at x.
class BrussJacobiProvider final : public Provider {
public:
    explicit BrussJacobiProvider(Brusselator1D& op) : op_(op) { a_.resize(4 * op.grid()); }
    void make(const double* x, const double*) override { op_.blocks(x, a_.p); }
    void apply(const double* r, double* z) override { brusselator_block_apply(op_.ctx(), a_.p, r, z, op_.grid()); }
    int kind() const override { return NUMA_GPU_PRECOND_BRUSS_JACOBI; }

private:
    Brusselator1D& op_;
    DeviceArray<double> a_;
};
}  // namespace

std::unique_ptr<Provider> make_bruss_jacobi_provider(Brusselator1D& op) {
    return std::make_unique<BrussJacobiProvider>(op);
}

// ============================================================================== Brusselator2D
Brusselator2D::Brusselator2D(Context& ctx, size_t n, const numa_brusselator2d_params& p)
    : NonlinearOp(ctx), n_(n), P_(p) {
    if (n < 3 || !(p.dt > 0.0) || !std::isfinite(p.dt) || !(p.Du >= 0.0) || !(p.Dv >= 0.0) || !std::isfinite(p.A) ||
        !std::isfinite(p.B) || !std::isfinite(p.Du) || !std::isfinite(p.Dv))
        throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "Brusselator2D requires n >= 3, dt > 0, D >= 0");
    if (n > 46340) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "Brusselator2D grid too large");
    prev_.resize(2 * n * n);
    dev_fill(ctx_, prev_.p, 0.0, 2 * n * n);
}

static B2Geom b2_geom(size_t n, const numa_brusselator2d_params& P) {
    B2Geom G;
    G.n = (int)n;
    const double h2inv = static_cast<double>(n) * static_cast<double>(n);
    G.invdt = 1.0 / P.dt;
    G.A = P.A;
    G.B = P.B;
    G.Bp1 = P.B + 1.0;
    G.c1 = G.invdt + (P.B + 1.0);
    G.duh = P.Du * h2inv;
    G.dvh = P.Dv * h2inv;
    return G;
}

void Brusselator2D::set_previous(const double* w) { dev_copy(ctx_, w, prev_.p, size()); }

void Brusselator2D::eval(const double* x, double* out, double*, double* norm_out) {
    const dim3 grid = b2_eval_grid((int)n_);
    if (grid.x * grid.y > (unsigned)kMaxRedBlocks) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "Brusselator2D grid too large");
    const B2Geom G = b2_geom(n_, P_);
    if (norm_out && fixed_sum_)
        launch_pdl(k_b2_eval<true, true>, grid, dim3(32, 8), 0, ctx_.stream, x, prev_.p, out, G, ctx_.red, norm_out);
    else if (norm_out)
        launch_pdl(k_b2_eval<true>, grid, dim3(32, 8), 0, ctx_.stream, x, prev_.p, out, G, ctx_.red, norm_out);
    else  // an evaluation without the norm (the reference-facing F) keeps the FP64 differences
        launch_pdl(k_b2_eval<false>, grid, dim3(32, 8), 0, ctx_.stream, x, prev_.p, out, G, ctx_.red, nullptr);
    ctx_.count_launch();
    ctx_.check_launch("Brusselator2D eval");
}

void Brusselator2D::bind(const double* x, const double*, int precision) {
    bound_x_ = x;
    bound_precision_ = precision;
    if (precision == NUMA_GPU_FP32) {
        const size_t nn = n_ * n_;
        coef32_.resize(nn);  // one float2 per point
        launch_pdl(k_b2_coef32, (unsigned)((nn + 255) / 256), 256, 0, ctx_.stream, x, nn,
                                                                          reinterpret_cast<float2*>(coef32_.p));
        ctx_.count_launch();
        ctx_.check_launch("Brusselator2D bind");
    }
}

void Brusselator2D::jvp_bound(const double* v, double* out) {
    if (bound_precision_ != NUMA_GPU_FP32) {
        jvp_at(bound_x_, v, out);
        return;
    }
    const B2Geom G = b2_geom(n_, P_);
    const B2Geom32 G32{(int)n_, (float)G.invdt, (float)G.B, (float)G.c1, (float)G.duh, (float)G.dvh};
    const dim3 grid((unsigned)((n_ + 31) / 32), (unsigned)((n_ + 7) / 8));
    launch_pdl(k_b2_jvp32<double>, grid, dim3(32, 8), 0, ctx_.stream, reinterpret_cast<const float2*>(coef32_.p), v, out,
                                                              G32);
    ctx_.count_launch();
    ctx_.check_launch("Brusselator2D jvp32");
}

void Brusselator2D::jvp_bound32(const float* v32, double* out) {
    if (bound_precision_ != NUMA_GPU_FP32)
        throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "Brusselator2D: no FP32 product bound");
    const B2Geom G = b2_geom(n_, P_);
    const B2Geom32 G32{(int)n_, (float)G.invdt, (float)G.B, (float)G.c1, (float)G.duh, (float)G.dvh};
    launch_pdl(k_b2_jvp32f<double>, b2_grid((int)n_), dim3(32, 8), 0, ctx_.stream,
               reinterpret_cast<const float2*>(coef32_.p), v32, out, G32);
    ctx_.count_launch();
    ctx_.check_launch("Brusselator2D jvp32 (fp32 input)");
}

void Brusselator2D::jvp_bound32f(const float* v32, float* out32) {
    if (bound_precision_ != NUMA_GPU_FP32)
        throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "Brusselator2D: no FP32 product bound");
    const B2Geom G = b2_geom(n_, P_);
    const B2Geom32 G32{(int)n_, (float)G.invdt, (float)G.B, (float)G.c1, (float)G.duh, (float)G.dvh};
    launch_pdl(k_b2_jvp32f<float>, b2_grid((int)n_), dim3(32, 8), 0, ctx_.stream,
               reinterpret_cast<const float2*>(coef32_.p), v32, out32, G32);
    ctx_.count_launch();
    ctx_.check_launch("Brusselator2D jvp32 (fp32 input and output)");
}

void Brusselator2D::jvp_at(const double* x, const double* v, double* out) {
    launch_pdl(k_b2_jvp, b2_grid((int)n_), dim3(32, 8), 0, ctx_.stream, x, v, out, b2_geom(n_, P_));
    ctx_.count_launch();
    ctx_.check_launch("Brusselator2D jvp");
}

void Brusselator2D::d2(const double* x, const double*, const double* v, double* out) {
    const size_t nn = n_ * n_;
    launch_pdl(k_bruss_d2, (unsigned)((nn + 255) / 256), 256, 0, ctx_.stream, x, v, out, nn);
    ctx_.count_launch();
    ctx_.check_launch("Brusselator2D d2");
}

// ============================================================================== BrussMG2D
struct BrussMG2D::Level {
    int n;
    double su, sv;
    DeviceArray<double> x, b, k;  // level pairs and blocks in the multigrid's precision
};

BrussMG2D::BrussMG2D(Context& ctx, size_t n, const numa_brusselator2d_params& p, int precision, int pre, int post)
    : ctx_(ctx), n0_(n), P_(p), precision_(precision), pre_(pre), post_(post) {
    if (n < 4 || n % 2 != 0) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "BrussMG2D needs an even n >= 4");
    if (n > 46340) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "BrussMG2D grid too large");
    if (pre < 1 || post < 1) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "BrussMG2D needs pre >= 1 and post >= 1");
    if (precision != NUMA_GPU_FP64 && precision != NUMA_GPU_FP32)
        throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "BrussMG2D precision must be FP64 or FP32");
    if (!(p.dt > 0.0) || !(p.Du >= 0.0) || !(p.Dv >= 0.0))
        throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "BrussMG2D requires dt > 0 and D >= 0");
    const size_t esz = precision == NUMA_GPU_FP64 ? 8 : 4;
    size_t m = n;
    for (;;) {
        auto L = std::make_unique<Level>();
        L->n = (int)m;
        L->su = p.Du * (static_cast<double>(m) * static_cast<double>(m));
        L->sv = p.Dv * (static_cast<double>(m) * static_cast<double>(m));
        const size_t mm = m * m;
        L->x.resize((2 * mm * esz + 7) / 8);
        L->b.resize((2 * mm * esz + 7) / 8);
        L->k.resize((4 * mm * esz + 7) / 8);
        levels_.push_back(std::move(L));
        if (m % 4 != 0 || m / 2 < 4) break;
        m /= 2;
    }
    // levels below the finest with n <= 64 (FP32) or n <= 32 (FP64) run as one block: x, b and K,
    // 8 (64^2 + 32^2 + ...) values, at most 175 KB of shared memory
    const int tail_max_n = precision == NUMA_GPU_FP64 ? kBmgTailMaxN / 2 : kBmgTailMaxN;
    for (size_t l = 1; l < levels_.size(); ++l)
        if (levels_[l]->n <= tail_max_n) {
            tail_first_ = (int)l;
            break;
        }
    if (tail_first_ > 0) {
        std::vector<TailLvl> d;
        size_t off = 0;
        for (size_t l = (size_t)tail_first_; l < levels_.size(); ++l) {
            const Level& L = *levels_[l];
            d.push_back(TailLvl{L.n, (int)off, L.k.p, LvlArgs<double>{L.n, L.su, L.sv, 4.0 * L.su, 4.0 * L.sv},
                                LvlArgs<float>{L.n, (float)L.su, (float)L.sv, (float)(4.0 * L.su),
                                               (float)(4.0 * L.sv)}});
            off += 8 * (size_t)L.n * L.n;
        }
        tail_count_ = (int)d.size();
        tail_smem_ = off * esz;
        tail_desc_.resize((d.size() * sizeof(TailLvl) + 7) / 8);
        NUMA_CUDA(cudaMemcpyAsync(tail_desc_.p, d.data(), d.size() * sizeof(TailLvl), cudaMemcpyHostToDevice,
                                  ctx_.stream));
        ctx_.sync();
        const int lim = precision == NUMA_GPU_FP64 ? set_dynamic_smem_limit(ctx_, k_bmg_tail<double>)
                                                   : set_dynamic_smem_limit(ctx_, k_bmg_tail<float>);
        if (tail_smem_ > (size_t)lim) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "BrussMG2D tail exceeds shared memory");
    }
}

BrussMG2D::~BrussMG2D() {
    if (coarse_exec_) cudaGraphExecDestroy(coarse_exec_);
}

template <class T>
static T* tp(DeviceArray<double>& a) {
    return reinterpret_cast<T*>(a.p);
}

void BrussMG2D::set_state(const double* w) {
    state_set_ = true;
    const size_t nn = n0_ * n0_;
    const double c1 = 1.0 / P_.dt + (P_.B + 1.0), c2 = 1.0 / P_.dt;
    const unsigned g = (unsigned)((nn + 255) / 256);
    if (precision_ == NUMA_GPU_FP64)
        launch_pdl(k_bmg_kfine<double>, g, 256, 0, ctx_.stream, w, (int)n0_, c1, c2, P_.B, tp<double>(levels_[0]->k));
    else
        launch_pdl(k_bmg_kfine<float>, g, 256, 0, ctx_.stream, w, (int)n0_, (float)c1, (float)c2, (float)P_.B,
                                                       tp<float>(levels_[0]->k));
    ctx_.count_launch();
    for (size_t l = 0; l + 1 < levels_.size(); ++l) {
        const int nc = levels_[l + 1]->n;
        const dim3 grid((unsigned)((nc + 31) / 32), (unsigned)((nc + 7) / 8));
        if (precision_ == NUMA_GPU_FP64)
            launch_pdl(k_bmg_krestrict<double>, grid, dim3(32, 8), 0, ctx_.stream, tp<double>(levels_[l]->k), levels_[l]->n,
                                                                          tp<double>(levels_[l + 1]->k));
        else
            launch_pdl(k_bmg_krestrict<float>, grid, dim3(32, 8), 0, ctx_.stream, tp<float>(levels_[l]->k), levels_[l]->n,
                                                                         tp<float>(levels_[l + 1]->k));
        ctx_.count_launch();
    }
    ctx_.check_launch("BrussMG2D set_state");
}

template <class T>
void BrussMG2D::cycle(size_t l) {
    Level& L = *levels_[l];
    const int n = L.n;
    const bool finest = l == 0;
    const bool coarsest = l + 1 == levels_.size();
    cudaStream_t s = ctx_.stream;
    T* X = tp<T>(L.x);
    T* Bv = tp<T>(L.b);
    const T* K = tp<T>(L.k);
    const LvlArgs<T> A{n, (T)L.su, (T)L.sv, (T)(4.0 * L.su), (T)(4.0 * L.sv)};
    const dim3 blk(32, 8);
    const dim3 pgrid((unsigned)((n / 2 + 31) / 32), (unsigned)((n + 7) / 8));
    const size_t nn = (size_t)n * n;
    if ((int)l == tail_first_) {
        launch_pdl(k_bmg_tail<T>, 1, kBmgTailThreads<T>, tail_smem_, s, reinterpret_cast<const TailLvl*>(tail_desc_.p), tail_count_, pre_,
                                                  post_, kBmgCoarsestSweeps, Bv, X);
        ctx_.count_launch();
        return;
    }
    if (coarsest) {
        if (finest) {
            if (r32_) launch_pdl(k_bmg_in<T, float>, (unsigned)((nn + 255) / 256), 256, 0, s, r32_, n, Bv);
            else launch_pdl(k_bmg_in<T>, (unsigned)((nn + 255) / 256), 256, 0, s, r0_, n, Bv);
            ctx_.count_launch();
        }
        if (nn <= (size_t)kBmgOneBlockPoints) {
            launch_pdl(k_bmg_coarsest<T>, 1, 1024, 0, s, X, Bv, K, A, kBmgCoarsestSweeps);
            ctx_.count_launch();
        } else {
            launch_pdl(k_bmg_pass<T, kBPassFirst>, pgrid, blk, 0, s, X, Bv, K, A, 0, nullptr, nullptr, nullptr);
            launch_pdl(k_bmg_pass<T, kBPassNormal>, pgrid, blk, 0, s, X, Bv, K, A, 1, nullptr, nullptr, nullptr);
            ctx_.count_launch(2);
            for (int k = 1; k < kBmgCoarsestSweeps; ++k) {
                launch_pdl(k_bmg_pass<T, kBPassNormal>, pgrid, blk, 0, s, X, Bv, K, A, 0, nullptr, nullptr, nullptr);
                launch_pdl(k_bmg_pass<T, kBPassNormal>, pgrid, blk, 0, s, X, Bv, K, A, 1, nullptr, nullptr, nullptr);
                ctx_.count_launch(2);
            }
        }
        if (finest) {
            launch_pdl(k_bmg_out<T>, (unsigned)((nn + 255) / 256), 256, 0, s, X, n, z0_);
            ctx_.count_launch();
        }
        return;
    }
    // pre-smoothing: colours 0, 1; the first pass starts from x = 0
    if (finest && r32_)
        launch_pdl(k_bmg_pass<T, kBPassFirst, float>, pgrid, blk, 0, s, X, Bv, K, A, 0, r32_, nullptr, nullptr);
    else
        launch_pdl(k_bmg_pass<T, kBPassFirst>, pgrid, blk, 0, s, X, Bv, K, A, 0, finest ? r0_ : nullptr, nullptr,
                   nullptr);
    launch_pdl(k_bmg_pass<T, kBPassNormal>, pgrid, blk, 0, s, X, Bv, K, A, 1, nullptr, nullptr, nullptr);
    ctx_.count_launch(2);
    for (int k = 1; k < pre_; ++k) {
        launch_pdl(k_bmg_pass<T, kBPassNormal>, pgrid, blk, 0, s, X, Bv, K, A, 0, nullptr, nullptr, nullptr);
        launch_pdl(k_bmg_pass<T, kBPassNormal>, pgrid, blk, 0, s, X, Bv, K, A, 1, nullptr, nullptr, nullptr);
        ctx_.count_launch(2);
    }
    Level& C = *levels_[l + 1];
    const int nc = C.n;
    launch_pdl(k_bmg_restrict<T>, dim3((unsigned)((nc + 15) / 16), (unsigned)((nc + 15) / 16)), dim3(16, 16), 0, s, 
        X, Bv, K, A, tp<T>(C.b));
    ctx_.count_launch();
    if (finest) coarse_cycle();
    else cycle<T>(l + 1);
    launch_pdl(k_bmg_prolong<T>, dim3((unsigned)((nc + 31) / 32), (unsigned)((nc + 7) / 8)), blk, 0, s, tp<T>(C.x), nc, X);
    ctx_.count_launch();
    // post-smoothing: colours 1, 0; the very last pass of the finest level writes z
    for (int k = 0; k < post_; ++k) {
        launch_pdl(k_bmg_pass<T, kBPassNormal>, pgrid, blk, 0, s, X, Bv, K, A, 1, nullptr, nullptr, nullptr);
        if (finest && k + 1 == post_)
            launch_pdl(k_bmg_pass<T, kBPassLast>, pgrid, blk, 0, s, X, Bv, K, A, 0, nullptr, z0_, z32_);
        else
            launch_pdl(k_bmg_pass<T, kBPassNormal>, pgrid, blk, 0, s, X, Bv, K, A, 0, nullptr, nullptr, nullptr);
        ctx_.count_launch(2);
    }
}

// Levels 1 and below as one CUDA graph: their arrays never move, and the blocks K are updated in
// place by set_state, so the graph captured on first use stays valid.
void BrussMG2D::coarse_cycle() {
    if (!coarse_exec_) {
        std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
        const uint64_t before = ctx_.launches;
        NUMA_CUDA(cudaStreamBeginCapture(ctx_.stream, cudaStreamCaptureModeThreadLocal));
        cudaGraph_t graph = nullptr;
        try {
            if (precision_ == NUMA_GPU_FP64) cycle<double>(1);
            else cycle<float>(1);
        } catch (...) {
            cudaStreamEndCapture(ctx_.stream, &graph);
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            throw;
        }
        NUMA_CUDA(cudaStreamEndCapture(ctx_.stream, &graph));
        const cudaError_t e = cudaGraphInstantiate(&coarse_exec_, graph, 0);
        cudaGraphDestroy(graph);
        NUMA_CUDA(e);
        coarse_kernels_ = ctx_.launches - before;
        ctx_.launches = before;
    }
    NUMA_CUDA(cudaGraphLaunch(coarse_exec_, ctx_.stream));
    ctx_.count_launch(static_cast<unsigned>(coarse_kernels_));
}

// Average duration of one colour pass on the finest level (the V-cycle's dominant kernel), over
// reps back-to-back launches timed with CUDA events on the context's stream; the blocks must have
// been set.
double BrussMG2D::time_finest_pass(int reps) {
    if (!state_set_) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "BrussMG2D: set_state before timing");
    Level& L = *levels_[0];
    const int n = L.n;
    const LvlArgs<double> A64{n, L.su, L.sv, 4.0 * L.su, 4.0 * L.sv};
    const LvlArgs<float> A32{n, (float)L.su, (float)L.sv, (float)(4.0 * L.su), (float)(4.0 * L.sv)};
    const dim3 blk(32, 8), pgrid((unsigned)((n / 2 + 31) / 32), (unsigned)((n + 7) / 8));
    const size_t esz = precision_ == NUMA_GPU_FP64 ? 8 : 4;
    NUMA_CUDA(cudaMemsetAsync(L.x.p, 0, 2 * (size_t)n * n * esz, ctx_.stream));
    NUMA_CUDA(cudaMemsetAsync(L.b.p, 0, 2 * (size_t)n * n * esz, ctx_.stream));
    cudaEvent_t a, b;
    NUMA_CUDA(cudaEventCreate(&a));
    NUMA_CUDA(cudaEventCreate(&b));
    auto launch = [&](int colour) {
        if (precision_ == NUMA_GPU_FP64)
            launch_pdl(k_bmg_pass<double, kBPassNormal>, pgrid, blk, 0, ctx_.stream, tp<double>(L.x),
                       tp<double>(L.b), tp<double>(L.k), A64, colour, nullptr, nullptr, nullptr);
        else
            launch_pdl(k_bmg_pass<float, kBPassNormal>, pgrid, blk, 0, ctx_.stream, tp<float>(L.x), tp<float>(L.b),
                       tp<float>(L.k), A32, colour, nullptr, nullptr, nullptr);
    };
    launch(0);
    NUMA_CUDA(cudaEventRecord(a, ctx_.stream));
    for (int r = 0; r < reps; ++r) launch(r & 1);
    NUMA_CUDA(cudaEventRecord(b, ctx_.stream));
    NUMA_CUDA(cudaEventSynchronize(b));
    float ms = 0.f;
    NUMA_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    ctx_.count_launch(reps + 1);
    ctx_.check_launch("BrussMG2D time_finest_pass");
    return reps > 0 ? ms / reps : 0.0;
}

void BrussMG2D::apply32(const double* r, float* z32) {
    if (!supports_out32()) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "BrussMG2D: no FP32 output for this hierarchy");
    z32_ = z32;
    try {
        apply(r, nullptr);
    } catch (...) {
        z32_ = nullptr;
        throw;
    }
    z32_ = nullptr;
}

void BrussMG2D::apply32f(const float* r32, float* z32) {
    if (!supports_out32()) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "BrussMG2D: no FP32 output for this hierarchy");
    r0_ = nullptr;
    r32_ = r32;
    z0_ = nullptr;
    z32_ = z32;
    try {
        cycle<float>(0);
    } catch (...) {
        r32_ = nullptr;
        z32_ = nullptr;
        throw;
    }
    r32_ = nullptr;
    z32_ = nullptr;
    ctx_.check_launch("BrussMG2D apply32f");
}

void BrussMG2D::apply(const double* r, double* z) {
    const size_t N = size();
    // the finest pass reads r while the last one writes z: an aliased call goes through a copy
    const double* rin = r;
    if (r == z) {
        alias_.resize(N);
        dev_copy(ctx_, r, alias_.p, N);
        rin = alias_.p;
    }
    r0_ = rin;
    z0_ = z;
    if (precision_ == NUMA_GPU_FP64) cycle<double>(0);
    else cycle<float>(0);
    ctx_.check_launch("BrussMG2D apply");
}

namespace {
// Provider over BrussMG2D: make(x) sets the blocks at the Newton iterate.
class BrussMGProvider final : public Provider {
public:
    BrussMGProvider(Context& ctx, size_t n, const numa_brusselator2d_params& p, int precision, int pre, int post)
        : mg_(ctx, n, p, precision, pre, post) {}
    void make(const double* x, const double*) override { mg_.set_state(x); }
    void apply(const double* r, double* z) override { mg_.apply(r, z); }
    // the FP32 cycle can hand its result over unwidened
    bool has_apply32() const override { return mg_.supports_out32(); }
    void apply32(const double* r, float* z32) override { mg_.apply32(r, z32); }
    bool has_apply32f() const override { return mg_.supports_out32(); }
    void apply32f(const float* r32, float* z32) override { mg_.apply32f(r32, z32); }
    int kind() const override { return NUMA_GPU_PRECOND_BRUSS_MG; }

private:
    BrussMG2D mg_;
};
}  // namespace

std::unique_ptr<Provider> make_bruss_mg_provider(Context& ctx, size_t n, const numa_brusselator2d_params& p,
                                                 int precision, int pre, int post) {
    return std::make_unique<BrussMGProvider>(ctx, n, p, precision, pre, post);
}

}  // namespace numa::gpu
