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
// a[(N+1)/2 + (L >> 1)].  A colour pass then reads and writes its own colour contiguously, and
// because every point of a pass has the same parity c, each neighbour (all of the other colour)
// sits at a fixed offset from the point's own index m = L >> 1:
//     k-1: m + c - 1        k+1: m + c
//     j-1: m + c - hn - 1   j+1: m + c + hn      (hn = (n - 1) / 2)
//     i-1: m + c - hP - 1   i+1: m + c + hP      (hP = (n^2 - 1) / 2)
// so a pass costs a handful of integer instructions per point.  Indices are 32-bit: the host
// uses this layout only for levels with N < 2^31.  Even n (only ever a coarsest level) keeps
// the natural layout.
struct Split {
    int n, half, hn, hP;  // half = (N + 1) / 2 = number of colour-0 points
};

inline Split make_split(int n) {
    const long long N = (long long)n * n * n;
    return Split{n, (int)((N + 1) / 2), (n - 1) / 2, (int)(((long long)n * n - 1) / 2)};
}

__device__ __forceinline__ int split_at(int L, int half) { return (L >> 1) + (L & 1) * half; }

enum SplitPass { kPassFull = 0, kPassFirst = 1, kPassLastZ = 2 };

// One colour pass of red-black Gauss-Seidel on the split layout, with the per-point arithmetic
// of k_rbgs<float> (b h^2 plus the six neighbours in the order i-1, i+1, j-1, j+1, k-1, k+1, then
// / 6).  A thread owns the k-pair {2kk, 2kk+1} of row j and marches over ICH planes; its point of
// colour c alternates between the two members from plane to plane.  The colour halves are
// separate restrict pointers (they never overlap), so the loads of all ICH planes can be in
// flight together.
//   kPassFirst: x is zero before the pass, x = bs / 6.
//   kPassLastZ: the final pass of the cycle: x is not stored; z (FP64, natural layout) receives
//               both members of the pair (the other member holds its value from the previous pass).
template <int MODE, int ICH>
__global__ void __launch_bounds__(BX* BY) k_pass_split(float* __restrict__ own, const float* __restrict__ oth,
                                                       const float* __restrict__ bown, double* __restrict__ z,
                                                       Split g, int c) {
    const int kk = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int n = g.n;
    if (j >= n || 2 * kk >= n) return;
    const int i0 = blockIdx.z * ICH;
    const int P = n * n;
    const int o_km = c - 1, o_kp = c, o_jm = c - g.hn - 1, o_jp = c + g.hn, o_im = c - g.hP - 1, o_ip = c + g.hP;
    const bool jlo = j > 0, jhi = j + 1 < n;
    int k = 2 * kk + ((i0 + j + c) & 1);
    int L = (i0 * n + j) * n + k;
#pragma unroll
    for (int s = 0; s < ICH; ++s) {
        const int i = i0 + s;
        if (i >= n) break;
        const int m = L >> 1;
        const bool valid = k < n;
        if (MODE == kPassLastZ) {
            const int ko = k ^ 1;
            if (ko < n) z[L - k + ko] = f32_to_f64(oth[m + (ko > k ? o_kp : o_km)]);
        }
        if (valid) {
            float v;
            if (MODE == kPassFirst) {
                v = div6(bown[m]);
            } else {
                float acc = bown[m], t;
                t = 0.0f;
                if (i > 0) t = oth[m + o_im];
                acc = acc + t;
                t = 0.0f;
                if (i + 1 < n) t = oth[m + o_ip];
                acc = acc + t;
                t = 0.0f;
                if (jlo) t = oth[m + o_jm];
                acc = acc + t;
                t = 0.0f;
                if (jhi) t = oth[m + o_jp];
                acc = acc + t;
                t = 0.0f;
                if (k > 0) t = oth[m + o_km];
                acc = acc + t;
                t = 0.0f;
                if (k + 1 < n) t = oth[m + o_kp];
                acc = acc + t;
                v = div6(acc);
            }
            if (MODE == kPassLastZ) z[L] = f32_to_f64(v);
            else own[m] = v;
        }
        const int kn = k ^ 1;
        L += P + (kn - k);
        k = kn;
    }
}

// Launches one colour pass on a split level: planes per thread 4 above 63 points, else 1.
template <int MODE>
inline void launch_pass_split(float* x, const float* bs, double* z, const Split& g, int c, cudaStream_t st) {
    float* own = x + (c ? g.half : 0);
    const float* oth = x + (c ? 0 : g.half);
    const float* bown = bs + (c ? g.half : 0);
    const int n = g.n;
    const dim3 blk(BX, BY);
    if (n >= 64) {
        const dim3 grid(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, (n + 3) / 4);
        k_pass_split<MODE, 4><<<grid, blk, 0, st>>>(own, oth, bown, z, g, c);
    } else {
        const dim3 grid(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, n);
        k_pass_split<MODE, 1><<<grid, blk, 0, st>>>(own, oth, bown, z, g, c);
    }
}

// r (natural layout) = b - h^-2 (6x - sum of neighbours) with x and b split: the order of
// k_residual (6x, then - i-1, - i+1, - j-1, - j+1, - k-1, - k+1).  A thread owns the k-pair
// {2kk, 2kk+1} of row j (colours cA and 1 - cA) and marches over ichunk planes.
__global__ void __launch_bounds__(BX* BY) k_residual_split(const float* __restrict__ x, const float* __restrict__ b,
                                                           float* __restrict__ r, Split g, int ichunk, float h2inv) {
    const int kk = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int n = g.n;
    if (j >= n || 2 * kk >= n) return;
    const int i0 = blockIdx.z * ichunk;
    const int i1 = min(i0 + ichunk, n);
    const int P = n * n;
    const bool jlo = j > 0, jhi = j + 1 < n, hasB = 2 * kk + 1 < n, kloA = kk > 0, khiB = 2 * kk + 2 < n;
    int LA = (i0 * n + j) * n + 2 * kk;
    for (int i = i0; i < i1; ++i, LA += P) {
        const int cA = (i + j) & 1, cB = cA ^ 1;
        const bool ilo = i > 0, ihi = i + 1 < n;
        // member A: k = 2kk, colour cA; its other-colour neighbours live in half cB
        const float* ownA = x + (cA ? g.half : 0);
        const float* othA = x + (cA ? 0 : g.half);
        const int mA = LA >> 1;
        const float xa = ownA[mA];
        float xb = 0.0f;
        if (hasB) xb = othA[mA + cA];  // member B (k = 2kk + 1) lives in A's other half
        {
            float s = 6.0f * xa, t;
            t = 0.0f;
            if (ilo) t = othA[mA + cA - g.hP - 1];
            s = s - t;
            t = 0.0f;
            if (ihi) t = othA[mA + cA + g.hP];
            s = s - t;
            t = 0.0f;
            if (jlo) t = othA[mA + cA - g.hn - 1];
            s = s - t;
            t = 0.0f;
            if (jhi) t = othA[mA + cA + g.hn];
            s = s - t;
            t = 0.0f;
            if (kloA) t = othA[mA + cA - 1];
            s = s - t;
            s = s - xb;
            r[LA] = b[(cA ? g.half : 0) + mA] - h2inv * s;
        }
        if (hasB) {
            const int LB = LA + 1, mB = LB >> 1;
            const float* othB = ownA;  // B's other colour is cA
            float s = 6.0f * xb, t;
            t = 0.0f;
            if (ilo) t = othB[mB + cB - g.hP - 1];
            s = s - t;
            t = 0.0f;
            if (ihi) t = othB[mB + cB + g.hP];
            s = s - t;
            t = 0.0f;
            if (jlo) t = othB[mB + cB - g.hn - 1];
            s = s - t;
            t = 0.0f;
            if (jhi) t = othB[mB + cB + g.hn];
            s = s - t;
            s = s - xa;
            t = 0.0f;
            if (khiB) t = othB[mB + cB];
            s = s - t;
            r[LB] = b[(cB ? g.half : 0) + mB] - h2inv * s;
        }
    }
}

// Restriction from a natural-layout fine residual into a split coarse level (odd nc): the
// 27-point sum of k_restrict in the same order, b and b h^2 stored split.  FIRST_X: also the
// coarse level's first smoothing pass (colour 0 from x = 0: x = bs / 6), which the cycle then
// skips.
template <bool FIRST_X>
__global__ void __launch_bounds__(BX* BY) k_restrict_split(const float* __restrict__ rf, float* __restrict__ bc,
                                                           float* __restrict__ bsc, float* __restrict__ xc, int nf,
                                                           int nc, int halfc, float inv_c) {
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
            const float* row = rf + (fi * nf + fj) * nf + 2 * K;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (2 * K + c >= nf) continue;
                acc = __fmaf_rn(wab * w[c], row[c], acc);
            }
        }
    }
    const int Lc = (I * nc + J) * nc + K;
    const int q = split_at(Lc, halfc);
    const float bsv = acc * inv_c;
    bc[q] = acc;
    bsc[q] = bsv;
    if (FIRST_X && !(Lc & 1)) xc[q] = div6(bsv);
}

// One fine point of a prolongation cell: x_f += sum over the present coarse neighbours (in the
// order i, j, k of k_prolong) of w * X, with w = (A ? 1 : 1/2)(B ? 1 : 1/2)(C ? 1 : 1/2).
// X[di][dj][dk] holds the coarse values at (I - 1 + di, J - 1 + dj, K - 1 + dk); pr*[d] tells
// whether that coarse index exists.
template <int A, int B, int C>
__device__ __forceinline__ void prolong_point(const float (&X)[2][2][2], const bool (&pi)[2], const bool (&pj)[2],
                                              const bool (&pk)[2], float* __restrict__ xf, int I, int J, int K,
                                              int nf, int halff) {
    const float w = (A ? 1.0f : 0.5f) * (B ? 1.0f : 0.5f) * (C ? 1.0f : 0.5f);
    float acc = 0.0f;
#pragma unroll
    for (int di = A; di < 2; ++di) {
        if (!pi[di]) continue;
#pragma unroll
        for (int dj = B; dj < 2; ++dj) {
            if (!pj[dj]) continue;
#pragma unroll
            for (int dk = C; dk < 2; ++dk) {
                if (!pk[dk]) continue;
                acc = __fmaf_rn(w, X[di][dj][dk], acc);
            }
        }
    }
    const int L = ((2 * I + A) * nf + 2 * J + B) * nf + 2 * K + C;
    float* e = xf + split_at(L, halff);
    *e = *e + acc;
}

// Fine x += trilinear interpolation of coarse x (k_prolong's arithmetic) on a split fine level.
// A thread owns the coarse cell (I, J, K), I, J, K in [0, nc], i.e. the fine points
// (2I + a, 2J + b, 2K + c), a, b, c in {0, 1}, inside the grid; it loads the eight coarse values
// around the cell once.  ALL = false: only the colour-0 fine points ((a + b + c) even), the only
// ones the first post-smoothing pass reads.  The coarse level is split (odd nc) or natural.
template <bool SPLIT_C, bool ALL>
__global__ void __launch_bounds__(BX* BY) k_prolong_split(const float* __restrict__ xc, float* __restrict__ xf,
                                                          int nc, int halfc, int nf, int halff) {
    const int K = blockIdx.x * BX + threadIdx.x;
    const int J = blockIdx.y * BY + threadIdx.y;
    const int I = blockIdx.z;
    if (K > nc || J > nc) return;
    const bool pi[2] = {I >= 1, I < nc}, pj[2] = {J >= 1, J < nc}, pk[2] = {K >= 1, K < nc};
    float X[2][2][2];
#pragma unroll
    for (int di = 0; di < 2; ++di)
#pragma unroll
        for (int dj = 0; dj < 2; ++dj)
#pragma unroll
            for (int dk = 0; dk < 2; ++dk) {
                float v = 0.0f;
                if (pi[di] && pj[dj] && pk[dk]) {
                    const int Lc = ((I - 1 + di) * nc + J - 1 + dj) * nc + K - 1 + dk;
                    v = xc[SPLIT_C ? split_at(Lc, halfc) : Lc];
                }
                X[di][dj][dk] = v;
            }
    const bool ia = I < nc, jb = J < nc, kc = K < nc;  // fine index 2I + 1 inside the grid
    prolong_point<0, 0, 0>(X, pi, pj, pk, xf, I, J, K, nf, halff);
    if (jb && kc) prolong_point<0, 1, 1>(X, pi, pj, pk, xf, I, J, K, nf, halff);
    if (ia && kc) prolong_point<1, 0, 1>(X, pi, pj, pk, xf, I, J, K, nf, halff);
    if (ia && jb) prolong_point<1, 1, 0>(X, pi, pj, pk, xf, I, J, K, nf, halff);
    if (ALL) {
        if (kc) prolong_point<0, 0, 1>(X, pi, pj, pk, xf, I, J, K, nf, halff);
        if (jb) prolong_point<0, 1, 0>(X, pi, pj, pk, xf, I, J, K, nf, halff);
        if (ia) prolong_point<1, 0, 0>(X, pi, pj, pk, xf, I, J, K, nf, halff);
        if (ia && jb && kc) prolong_point<1, 1, 1>(X, pi, pj, pk, xf, I, J, K, nf, halff);
    }
}

// b32 = RN32(r), bs32 = RN32(b32 * inv) into the split layout at the finest level; WRITE_X: also
// the cycle's first smoothing pass (colour 0 from x = 0: x = bs / 6).  Thread t handles the
// natural pair L = 2t (colour 0, index t) and L = 2t + 1 (colour 1, index half + t).
template <bool WRITE_X>
__global__ void k_scale_in32_split(const double* __restrict__ r, float* __restrict__ b, float* __restrict__ bs,
                                   float* __restrict__ x, float inv, int N, int half) {
    const int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < half; t += stride) {
        const int L = 2 * t;
        const float v0 = f64_to_f32(r[L]);
        const float s0 = v0 * inv;
        b[t] = v0;
        bs[t] = s0;
        if (WRITE_X) x[t] = div6(s0);
        if (L + 1 < N) {
            const float v1 = f64_to_f32(r[L + 1]);
            b[half + t] = v1;
            bs[half + t] = v1 * inv;
        }
    }
}

// z (FP64, natural) = x (FP32, split)
__global__ void k_to64_split(const float* __restrict__ x, double* __restrict__ z, int N, int half) {
    const int stride = gridDim.x * blockDim.x;
    for (int L = blockIdx.x * blockDim.x + threadIdx.x; L < N; L += stride) z[L] = f32_to_f64(x[split_at(L, half)]);
}

}  // namespace
}  // namespace numa::gpu
