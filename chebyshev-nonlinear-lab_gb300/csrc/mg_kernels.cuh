// mg_kernels.cuh — the geometric-multigrid kernels shared by the V-cycle implementations
// (poisson_mg.cu and the fixed-scratch variant).  See poisson_mg.cu for the algorithm and its
// reference citations.  Everything here has internal linkage: each including file gets its own
// copy of the kernels it launches.
#pragma once

#include "numa_internal.hpp"

namespace numa::gpu {
namespace {

constexpr int MG_BX = 32, MG_BY = 8;
constexpr int BX = MG_BX, BY = MG_BY;

template <class T> __device__ __forceinline__ T zero() { return T(0); }

// One colour pass of red-black Gauss-Seidel.  FIRST: x is zero before this pass, so the update
// is bs / 6.  OUT_Z: also store the result as FP64 into z.
template <class T, bool FIRST, bool OUT_Z>
__global__ void __launch_bounds__(BX* BY) k_rbgs(T* __restrict__ x, const T* __restrict__ bs, double* __restrict__ z,
                                                 int n, int colour) {
    const int kk = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int i = blockIdx.z;
    if (j >= n) return;
    const int k = 2 * kk + ((i + j + colour) & 1);
    if (k >= n) return;
    const size_t plane = (size_t)n * n;
    const size_t p = ((size_t)i * n + j) * n + k;
    T v;
    if (FIRST) {
        v = div6(bs[p]);
    } else {
        T acc = bs[p];
        acc = acc + ((i > 0) ? x[p - plane] : zero<T>());
        acc = acc + ((i + 1 < n) ? x[p + plane] : zero<T>());
        acc = acc + ((j > 0) ? x[p - n] : zero<T>());
        acc = acc + ((j + 1 < n) ? x[p + n] : zero<T>());
        acc = acc + ((k > 0) ? x[p - 1] : zero<T>());
        acc = acc + ((k + 1 < n) ? x[p + 1] : zero<T>());
        v = div6(acc);
    }
    x[p] = v;
    if (OUT_Z) z[p] = (sizeof(T) == 4) ? f32_to_f64((float)v) : (double)v;
}

// r = b - h^-2 (6x - sum of neighbours) (poisson_mg.hpp:128-149), marching in i.
template <class T>
__global__ void __launch_bounds__(BX* BY) k_residual(const T* __restrict__ x, const T* __restrict__ b,
                                                     T* __restrict__ r, int n, int ichunk, T h2inv) {
    const int k = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int i0 = blockIdx.z * ichunk;
    const int i1 = min(i0 + ichunk, n);
    if (k >= n || j >= n) return;
    const size_t plane = (size_t)n * n;
    size_t p = ((size_t)i0 * n + j) * n + k;
    T below = (i0 > 0) ? x[p - plane] : zero<T>();
    T cur = x[p];
    for (int i = i0; i < i1; ++i) {
        const T above = (i + 1 < n) ? x[p + plane] : zero<T>();
        T s = T(6) * cur;
        s = s - below;
        s = s - above;
        s = s - ((j > 0) ? x[p - n] : zero<T>());
        s = s - ((j + 1 < n) ? x[p + n] : zero<T>());
        s = s - ((k > 0) ? x[p - 1] : zero<T>());
        s = s - ((k + 1 < n) ? x[p + 1] : zero<T>());
        r[p] = b[p] - h2inv * s;
        below = cur;
        cur = above;
        p += plane;
    }
}

__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// Coarse b = sum over the 27 fine points 2I+{0,1,2} of (w_a w_b w_c) r, weights (1/4,1/2,1/4),
// summed a (i) outer, b (j), c (k) inner (poisson_mg.hpp:152-188).  Each weight product is a
// power of two, so w*r is exact and the FMA equals the reference's multiply-then-add.  Also
// stores bs = b * inv_c for the smoother.
template <class T>
__global__ void __launch_bounds__(BX* BY) k_restrict(const T* __restrict__ rf, T* __restrict__ bc,
                                                     T* __restrict__ bsc, int nf, int nc, double inv_c) {
    const int K = blockIdx.x * BX + threadIdx.x;
    const int J = blockIdx.y * BY + threadIdx.y;
    const int I = blockIdx.z;
    if (K >= nc || J >= nc) return;
    const T w[3] = {T(0.25), T(0.5), T(0.25)};
    T acc = zero<T>();
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int fi = 2 * I + a;
        if (fi >= nf) continue;
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const int fj = 2 * J + b;
            if (fj >= nf) continue;
            const T wab = w[a] * w[b];
            const T* row = rf + ((size_t)fi * nf + fj) * nf;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const int fk = 2 * K + c;
                if (fk >= nf) continue;
                acc = fma_t(wab * w[c], row[fk], acc);
            }
        }
    }
    const size_t q = ((size_t)I * nc + J) * nc + K;
    bc[q] = acc;
    bsc[q] = acc * (T)inv_c;  // FP64: the reference's b * inv; FP32: RN32(b * RN32(inv))
}

// 1D interpolation stencil (poisson_mg.hpp:191-220).
__device__ __forceinline__ int interp(int f, int nc, int (&idx)[2]) {
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

// Fine x += trilinear interpolation of coarse x (poisson_mg.hpp:222-260).  COLOUR0_ONLY:
// only points with (i+j+k) even.  Weights: 1 for an odd index, 1/2 per term for an even one;
// products are powers of two, so w * xc is exact and the FMA equals the reference's sum.
template <class T, bool COLOUR0_ONLY>
__global__ void __launch_bounds__(BX* BY) k_prolong(const T* __restrict__ xc, T* __restrict__ xf, int nc, int nf) {
    const int t = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int i = blockIdx.z;
    if (j >= nf) return;
    const int k = COLOUR0_ONLY ? 2 * t + ((i + j) & 1) : t;
    if (k >= nf) return;
    int ci[2], cj[2], ck[2];
    const int ni = interp(i, nc, ci), nj = interp(j, nc, cj), nk = interp(k, nc, ck);
    const T wi = (ni == 1 && (i & 1)) ? T(1) : T(0.5);
    const T wj = (nj == 1 && (j & 1)) ? T(1) : T(0.5);
    const T wk = (nk == 1 && (k & 1)) ? T(1) : T(0.5);
    T acc = zero<T>();
    for (int a = 0; a < ni; ++a)
        for (int b = 0; b < nj; ++b) {
            const T* row = xc + ((size_t)ci[a] * nc + cj[b]) * nc;
            for (int c = 0; c < nk; ++c) acc = fma_t(wi * wj * wk, row[ck[c]], acc);
        }
    const size_t p = ((size_t)i * nf + j) * nf + k;
    xf[p] = xf[p] + acc;
}

// bs = r * inv at the finest FP64 level.
__global__ void k_scale_in64(const double* __restrict__ r, double* __restrict__ bs, double inv, size_t N) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) bs[p] = r[p] * inv;
}

// b32 = RN32(r), bs32 = RN32(b32 * RN32(inv)) at the finest FP32 level (conversions in integer
// arithmetic: no FP64 instruction).
__global__ void k_scale_in32(const double* __restrict__ r, float* __restrict__ b, float* __restrict__ bs, float inv,
                             size_t N) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) {
        const float v = f64_to_f32(r[p]);
        b[p] = v;
        bs[p] = v * inv;
    }
}

__global__ void k_to64(const float* __restrict__ x, double* __restrict__ z, size_t N) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) z[p] = f32_to_f64(x[p]);
}

// Coarsest level with one point: x = b / (6 h^-2) (poisson_mg.hpp:267-269).
template <class T>
__global__ void k_single(const T* __restrict__ b, T* __restrict__ x, double* __restrict__ z, double six_h2inv) {
    const T v = (T)((double)b[0] / six_h2inv);
    x[0] = v;
    if (z) z[0] = (double)v;
}

}  // namespace
}  // namespace numa::gpu

namespace numa::gpu {
namespace {

// ------------------------------------------------------------------------------------------
// Fused red-black Gauss-Seidel sweep in FP32 (both colours in one kernel, one read of x and of
// b h^2 and one write of x per point) for the mixed-precision V-cycle, whose kernels are bound
// by HBM bandwidth.  The same arithmetic per point as two k_rbgs<float> passes (the colour-c0
// update, then the colour-c1 update from the new c0 values), so the result is identical.
//
// A block owns a 32 (k) x 16 (j) tile and a chunk of i planes and streams the planes through a
// ring of four shared-memory slots, each holding one plane of the tile with a 2-point halo:
//   load raw plane p+1; update colour c0 of plane p over the tile plus a 1-point halo (its
//   in-plane neighbours reach 2 points out); update colour c1 of plane p-1 over the tile (all
//   its neighbours are colour-c0 values now final); store plane p-1.
// The sweep is out of place (xin -> xout): blocks read halo planes that neighbouring blocks
// write, so reads must see the values from before the sweep.  FIRST: xin is zero (no loads).
constexpr int SW_TK = 32, SW_TJ = 16;
constexpr int SW_SK = SW_TK + 4, SW_SJ = SW_TJ + 4;
constexpr int SW_PLANE = SW_SK * SW_SJ;
constexpr int SW_THREADS = 256;

template <bool FIRST, bool OUT_X, bool OUT_Z>
__global__ void __launch_bounds__(SW_THREADS) k_rbgs_sweep32(const float* __restrict__ xin, float* __restrict__ xout,
                                                            const float* __restrict__ bs, double* __restrict__ z,
                                                            int n, int c0, int ichunk) {
    __shared__ float P[4][SW_PLANE];
    const int tid = threadIdx.x;
    const int k0 = blockIdx.x * SW_TK, j0 = blockIdx.y * SW_TJ;
    const int ib = blockIdx.z * ichunk;
    const int ie = min(ib + ichunk, n);
    const int c1 = 1 - c0;
    const size_t plane = (size_t)n * n;
    auto slot = [](int p) { return (p + 8) & 3; };

    auto load = [&](int p) {
        float* S = P[slot(p)];
        const bool inside = !FIRST && p >= 0 && p < n;
        for (int e = tid; e < SW_PLANE; e += SW_THREADS) {
            const int sj = e / SW_SK, sk = e - sj * SW_SK;
            const int j = j0 - 2 + sj, k = k0 - 2 + sk;
            float v = 0.0f;
            if (inside && j >= 0 && j < n && k >= 0 && k < n) v = xin[(size_t)p * plane + (size_t)j * n + k];
            S[e] = v;
        }
    };
    // one Gauss-Seidel update at smem index e of plane p (neighbours in the slots of p-1, p, p+1)
    auto update = [&](int p, int j, int k) {
        const int e = (j - j0 + 2) * SW_SK + (k - k0 + 2);
        const float* Sm = P[slot(p - 1)];
        const float* Sp = P[slot(p + 1)];
        float* S = P[slot(p)];
        float acc = bs[(size_t)p * plane + (size_t)j * n + k];
        acc = acc + Sm[e];
        acc = acc + Sp[e];
        acc = acc + S[e - SW_SK];
        acc = acc + S[e + SW_SK];
        acc = acc + S[e - 1];
        acc = acc + S[e + 1];
        S[e] = div6(acc);
    };
    // colour c0 of plane p over the tile and a 1-point halo (rows j0-1 .. j0+16, 17 points a row)
    auto upd0 = [&](int p) {
        if (p < 0 || p >= n) return;
        constexpr int rows = SW_TJ + 2, per = (SW_TK + 2) / 2;
        for (int t = tid; t < rows * per; t += SW_THREADS) {
            const int r = t / per, q = t - r * per;
            const int j = j0 - 1 + r;
            const int k = k0 - 1 + ((c0 + p + j + k0 + 1) & 1) + 2 * q;
            if (j >= 0 && j < n && k >= 0 && k < n) update(p, j, k);
        }
    };
    // colour c1 of plane p over the tile (16 points a row, one per thread)
    auto upd1 = [&](int p) {
        const int r = tid / (SW_TK / 2), q = tid - r * (SW_TK / 2);
        const int j = j0 + r;
        const int k = k0 + ((c1 + p + j + k0) & 1) + 2 * q;
        if (j < n && k < n) update(p, j, k);
    };
    auto store = [&](int p) {
        const float* S = P[slot(p)];
        for (int e = tid; e < SW_TK * SW_TJ; e += SW_THREADS) {
            const int r = e / SW_TK, c = e - r * SW_TK;
            const int j = j0 + r, k = k0 + c;
            if (j < n && k < n) {
                const float v = S[(r + 2) * SW_SK + (c + 2)];
                const size_t g = (size_t)p * plane + (size_t)j * n + k;
                if (OUT_X) xout[g] = v;
                if (OUT_Z) z[g] = f32_to_f64(v);
            }
        }
    };

    load(ib - 2);
    load(ib - 1);
    load(ib);
    __syncthreads();
    upd0(ib - 1);
    __syncthreads();
    for (int p = ib; p <= ie; ++p) {
        load(p + 1);
        __syncthreads();
        upd0(p);
        __syncthreads();
        if (p - 1 >= ib) {
            upd1(p - 1);
            __syncthreads();
            store(p - 1);
        }
    }
}

}  // namespace
}  // namespace numa::gpu
