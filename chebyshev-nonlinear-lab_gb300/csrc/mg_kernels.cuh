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
// Colour-split FP32 layout (the mixed-precision cycle, levels of odd n).  For odd n the colour
// of point L = (i*n + j)*n + k is (i+j+k) & 1 = L & 1, so the level array is stored
// de-interleaved: colour-0 values at a[L >> 1] (the first (N+1)/2 floats), colour-1 values at
// a[(N+1)/2 + (L >> 1)].  A colour pass then reads and writes its own colour contiguously and
// finds each neighbour L +- 1, +- n, +- n^2 (all of the other colour) at (L +- d) >> 1 of the
// other half: every access is coalesced and no sector is read or written half-used, which the
// HBM-bound FP32 cycle needs.  Even n (only ever a coarsest level) keeps the natural layout.
__device__ __forceinline__ size_t split_index(size_t L, size_t N) { return (L & 1) ? (N + 1) / 2 + (L >> 1) : (L >> 1); }

// One colour pass on the split layout: the same arithmetic per point as k_rbgs<float>.
template <bool FIRST>
__global__ void __launch_bounds__(BX* BY) k_rbgs_split(float* __restrict__ x, const float* __restrict__ bs, int n,
                                                       int colour) {
    const int kk = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int i = blockIdx.z;
    if (j >= n) return;
    const int k = 2 * kk + ((i + j + colour) & 1);
    if (k >= n) return;
    const size_t plane = (size_t)n * n, N = plane * n, half = (N + 1) / 2;
    const size_t L = ((size_t)i * n + j) * n + k;
    const size_t m = L >> 1;
    float* own = x + (colour ? half : 0);
    const float* oth = x + (colour ? 0 : half);
    const float* bown = bs + (colour ? half : 0);
    float v;
    if (FIRST) {
        v = div6(bown[m]);
    } else {
        float acc = bown[m];
        acc = acc + ((i > 0) ? oth[(L - plane) >> 1] : 0.0f);
        acc = acc + ((i + 1 < n) ? oth[(L + plane) >> 1] : 0.0f);
        acc = acc + ((j > 0) ? oth[(L - n) >> 1] : 0.0f);
        acc = acc + ((j + 1 < n) ? oth[(L + n) >> 1] : 0.0f);
        acc = acc + ((k > 0) ? oth[(L - 1) >> 1] : 0.0f);
        acc = acc + ((k + 1 < n) ? oth[(L + 1) >> 1] : 0.0f);
        v = div6(acc);
    }
    own[m] = v;
}

// r (natural layout) = b - h^-2 (6x - sum) with x and b in the split layout, marching in i.
__global__ void __launch_bounds__(BX* BY) k_residual_split(const float* __restrict__ x, const float* __restrict__ b,
                                                           float* __restrict__ r, int n, int ichunk, float h2inv) {
    const int k = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int i0 = blockIdx.z * ichunk;
    const int i1 = min(i0 + ichunk, n);
    if (k >= n || j >= n) return;
    const size_t plane = (size_t)n * n, N = plane * n;
    auto at = [&](size_t L) { return x[split_index(L, N)]; };
    size_t L = ((size_t)i0 * n + j) * n + k;
    float below = (i0 > 0) ? at(L - plane) : 0.0f;
    float cur = at(L);
    for (int i = i0; i < i1; ++i) {
        const float above = (i + 1 < n) ? at(L + plane) : 0.0f;
        float s = 6.0f * cur;
        s = s - below;
        s = s - above;
        s = s - ((j > 0) ? at(L - n) : 0.0f);
        s = s - ((j + 1 < n) ? at(L + n) : 0.0f);
        s = s - ((k > 0) ? at(L - 1) : 0.0f);
        s = s - ((k + 1 < n) ? at(L + 1) : 0.0f);
        r[L] = b[split_index(L, N)] - h2inv * s;
        below = cur;
        cur = above;
        L += plane;
    }
}

// Restriction from a natural-layout fine residual into coarse b, b h^2 stored split (odd nc).
__global__ void __launch_bounds__(BX* BY) k_restrict_split(const float* __restrict__ rf, float* __restrict__ bc,
                                                           float* __restrict__ bsc, int nf, int nc, float inv_c) {
    const int K = blockIdx.x * BX + threadIdx.x;
    const int J = blockIdx.y * BY + threadIdx.y;
    const int I = blockIdx.z;
    if (K >= nc || J >= nc) return;
    const float w[3] = {0.25f, 0.5f, 0.25f};
    float acc = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int fi = 2 * I + a;
        if (fi >= nf) continue;
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) {
            const int fj = 2 * J + bb;
            if (fj >= nf) continue;
            const float wab = w[a] * w[bb];
            const float* row = rf + ((size_t)fi * nf + fj) * nf;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const int fk = 2 * K + c;
                if (fk >= nf) continue;
                acc = __fmaf_rn(wab * w[c], row[fk], acc);
            }
        }
    }
    const size_t Nc = (size_t)nc * nc * nc;
    const size_t q = split_index(((size_t)I * nc + J) * nc + K, Nc);
    bc[q] = acc;
    bsc[q] = acc * inv_c;
}

// Fine x += trilinear interpolation of coarse x (colour-0 fine points only, or all with ALL);
// the fine level is split, the coarse one split when nc is odd.
template <bool SPLIT_C, bool ALL>
__global__ void __launch_bounds__(BX* BY) k_prolong_split(const float* __restrict__ xc, float* __restrict__ xf, int nc,
                                                          int nf) {
    const int t = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int i = blockIdx.z;
    if (j >= nf) return;
    const int k = ALL ? t : 2 * t + ((i + j) & 1);
    if (k >= nf) return;
    int ci[2], cj[2], ck[2];
    const int ni = interp(i, nc, ci), nj = interp(j, nc, cj), nk = interp(k, nc, ck);
    const float wi = (ni == 1 && (i & 1)) ? 1.0f : 0.5f;
    const float wj = (nj == 1 && (j & 1)) ? 1.0f : 0.5f;
    const float wk = (nk == 1 && (k & 1)) ? 1.0f : 0.5f;
    const size_t Nc = (size_t)nc * nc * nc;
    float acc = 0.0f;
    for (int a = 0; a < ni; ++a)
        for (int bb = 0; bb < nj; ++bb) {
            const size_t row = ((size_t)ci[a] * nc + cj[bb]) * nc;
            for (int c = 0; c < nk; ++c) {
                const size_t Lc = row + ck[c];
                acc = __fmaf_rn(wi * wj * wk, xc[SPLIT_C ? split_index(Lc, Nc) : Lc], acc);
            }
        }
    const size_t L = ((size_t)i * nf + j) * nf + k;
    float* e = xf + split_index(L, (size_t)nf * nf * nf);
    *e = *e + acc;
}

// b32 = RN32(r), bs32 = RN32(b32 * RN32(inv)) into the split layout (finest odd level).
__global__ void k_scale_in32_split(const double* __restrict__ r, float* __restrict__ b, float* __restrict__ bs,
                                   float inv, size_t N) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t L = blockIdx.x * (size_t)blockDim.x + threadIdx.x; L < N; L += stride) {
        const float v = f64_to_f32(r[L]);
        const size_t q = split_index(L, N);
        b[q] = v;
        bs[q] = v * inv;
    }
}

// z (FP64, natural) = x (FP32, split)
__global__ void k_to64_split(const float* __restrict__ x, double* __restrict__ z, size_t N) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t L = blockIdx.x * (size_t)blockDim.x + threadIdx.x; L < N; L += stride)
        z[L] = f32_to_f64(x[split_index(L, N)]);
}

}  // namespace
}  // namespace numa::gpu
