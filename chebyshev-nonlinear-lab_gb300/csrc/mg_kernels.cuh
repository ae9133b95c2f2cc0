// mg_kernels.cuh — the geometric-multigrid kernels shared by the V-cycle implementations
// (poisson_mg.cu and the fixed-scratch variant).  See poisson_mg.cu for the algorithm and its
// reference citations.  Everything here has internal linkage: each including file gets its own
// copy of the kernels it launches.
#pragma once

#include <type_traits>
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
    pdl_wait();
    pdl_trigger();
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
    pdl_wait();
    pdl_trigger();
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
    pdl_wait();
    pdl_trigger();
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
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int i = blockIdx.z;
    if (j >= nf) return;
    const int k = COLOUR0_ONLY ? 2 * t + ((i + j) & 1) : t;
    if (k >= nf) return;
    int ci[2], cj[2], ck[2];
    const int ni = interp(i, nc, ci), nj = interp(j, nc, cj), nk = interp(k, nc, ck);
    // w = wi wj wk, each 1 (odd index) or 1/2: the power of two 2^-halves, picked without FP64 work
    const int halves = !(ni == 1 && (i & 1)) + !(nj == 1 && (j & 1)) + !(nk == 1 && (k & 1));
    const T w = halves == 0 ? T(1) : (halves == 1 ? T(0.5) : (halves == 2 ? T(0.25) : T(0.125)));
    T acc = zero<T>();
    for (int a = 0; a < ni; ++a)
        for (int b = 0; b < nj; ++b) {
            const T* row = xc + ((size_t)ci[a] * nc + cj[b]) * nc;
            for (int c = 0; c < nk; ++c) acc = fma_t(w, row[ck[c]], acc);
        }
    const size_t p = ((size_t)i * nf + j) * nf + k;
    xf[p] = xf[p] + acc;
}

// bs = r * inv at the finest FP64 level.
__global__ void k_scale_in64(const double* __restrict__ r, double* __restrict__ bs, double inv, size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) bs[p] = r[p] * inv;
}

// b32 = RN32(r), bs32 = RN32(b32 * RN32(inv)) at the finest FP32 level (conversions in integer
// arithmetic: no FP64 instruction).
// RT = double (an FP64 right-hand side, rounded here) or float (already FP32: copied as is)
template <class RT>
__global__ void k_scale_in32(const RT* __restrict__ r, float* __restrict__ b, float* __restrict__ bs, float inv,
                             size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) {
        const float v = f64_to_f32(r[p]);
        b[p] = v;
        bs[p] = v * inv;
    }
}

__global__ void k_to64(const float* __restrict__ x, double* __restrict__ z, size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) z[p] = f32_to_f64(x[p]);
}

// Coarsest level with one point: x = b / (6 h^-2) (poisson_mg.hpp:267-269).
template <class T>
__global__ void k_single(const T* __restrict__ b, T* __restrict__ x, double* __restrict__ z, double six_h2inv) {
    pdl_wait();
    pdl_trigger();
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
// colour c alternates between the two members from plane to plane.  The level arrays are padded
// (x by more than a colour plane on each side, b h^2 at the end), so every load is issued
// unconditionally: first all loads of the ICH planes, then the arithmetic, with a select putting
// +0.0 in place of a neighbour outside the grid.  The colour halves are separate restrict
// pointers (they never overlap).
//   kPassFirst: x is zero before the pass, x = bs / 6.
//   kPassLastZ: the final pass of the cycle: x is not stored; z (FP64, natural layout) receives
//               both members of the pair (the other member holds its value from the previous pass),
//               or z32 (FP32) the same values unwidened, for consumers that work in FP32.
//   NN > 0: the grid size is a compile-time constant, so every neighbour offset is an immediate of
//           the load instruction (one add per point forms the base m + c).
// The body takes its block coordinates as arguments, so that the batched form (below) can run it
// on one grid of a pool.
template <int MODE, int ICH, int NN>
__device__ __forceinline__ void pass_split_body(float* __restrict__ own, const float* __restrict__ oth,
                                                const float* __restrict__ bown, double* __restrict__ z, Split g,
                                                int c, float* __restrict__ z32, int bx, int by, int bz) {
    const int kk = bx * BX + threadIdx.x;
    const int j = by * BY + threadIdx.y;
    const int n = NN > 0 ? NN : g.n;
    if (j >= n || 2 * kk >= n) return;
    const int i0 = bz * ICH;
    const int P = n * n;
    const int hn = NN > 0 ? (NN - 1) / 2 : g.hn, hP = NN > 0 ? (NN * NN - 1) / 2 : g.hP;
    const bool jlo = j > 0, jhi = j + 1 < n;
    const int kA = 2 * kk + ((i0 + j + c) & 1);  // the point's k on planes i0, i0 + 2, ...
    const int LA = (i0 * n + j) * n + kA;
    float bv[ICH], v_im[ICH], v_ip[ICH], v_jm[ICH], v_jp[ICH], v_km[ICH], v_kp[ICH];
#pragma unroll
    for (int s = 0; s < ICH; ++s) {
        const int k = (s & 1) ? (kA ^ 1) : kA;
        const int L = LA + s * P + (k - kA);
        const int m = (i0 + s < n) ? (L >> 1) : 0;  // planes past the grid load harmlessly
        bv[s] = bown[m];
        if (MODE != kPassFirst) {
            const float* q = oth + (m + c);  // the neighbours at fixed offsets from here
            v_im[s] = q[-hP - 1];
            v_ip[s] = q[hP];
            v_jm[s] = q[-hn - 1];
            v_jp[s] = q[hn];
            v_km[s] = q[-1];
            v_kp[s] = q[0];
        }
    }
#pragma unroll
    for (int s = 0; s < ICH; ++s) {
        const int i = i0 + s;
        if (i >= n) break;
        const int k = (s & 1) ? (kA ^ 1) : kA;
        const int L = LA + s * P + (k - kA);
        const int m = L >> 1;
        if (MODE == kPassLastZ) {
            const int ko = k ^ 1;
            if (ko < n) {
                const float vo = ko > k ? v_kp[s] : v_km[s];
                if (z) z[L - k + ko] = f32_to_f64(vo);
                if (z32) z32[L - k + ko] = vo;
            }
        }
        if (k < n) {
            float v;
            if (MODE == kPassFirst) {
                v = div6(bv[s]);
            } else {
                float acc = bv[s];
                acc = acc + ((i > 0) ? v_im[s] : 0.0f);
                acc = acc + ((i + 1 < n) ? v_ip[s] : 0.0f);
                acc = acc + (jlo ? v_jm[s] : 0.0f);
                acc = acc + (jhi ? v_jp[s] : 0.0f);
                acc = acc + ((k > 0) ? v_km[s] : 0.0f);
                acc = acc + ((k + 1 < n) ? v_kp[s] : 0.0f);
                v = div6(acc);
            }
            if (MODE == kPassLastZ) {
                if (z) z[L] = f32_to_f64(v);
                if (z32) z32[L] = v;
            } else {
                own[m] = v;
            }
        }
    }
}

template <int MODE, int ICH, int NN>
__global__ void __launch_bounds__(BX* BY) k_pass_split(float* __restrict__ own, const float* __restrict__ oth,
                                                       const float* __restrict__ bown, double* __restrict__ z,
                                                       Split g, int c, float* __restrict__ z32 = nullptr) {
    pdl_wait();
    pdl_trigger();
    pass_split_body<MODE, ICH, NN>(own, oth, bown, z, g, c, z32, blockIdx.x, blockIdx.y, blockIdx.z);
}

// Launches one colour pass on a split level: planes per thread 4 above 63 points, else 1.
template <int MODE>
inline void launch_pass_split(float* x, const float* bs, double* z, const Split& g, int c, cudaStream_t st,
                              float* z32 = nullptr) {
    float* own = x + (c ? g.half : 0);
    const float* oth = x + (c ? 0 : g.half);
    const float* bown = bs + (c ? g.half : 0);
    const int n = g.n;
    const dim3 blk(BX, BY);
    if (n >= 64) {
        const dim3 grid(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, (n + 3) / 4);
        if (n == 255) launch_pdl(k_pass_split<MODE, 4, 255>, grid, blk, 0, st, own, oth, bown, z, g, c, z32);
        else if (n == 127) launch_pdl(k_pass_split<MODE, 4, 127>, grid, blk, 0, st, own, oth, bown, z, g, c, z32);
        else launch_pdl(k_pass_split<MODE, 4, 0>, grid, blk, 0, st, own, oth, bown, z, g, c, z32);
    } else {
        const dim3 grid(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, n);
        launch_pdl(k_pass_split<MODE, 1, 0>, grid, blk, 0, st, own, oth, bown, z, g, c, z32);
    }
}

// r (natural layout) = b - h^-2 (6x - sum of neighbours) with x and b split: the order of
// k_residual (6x, then - i-1, - i+1, - j-1, - j+1, - k-1, - k+1).  A thread owns the k-pair
// {2kk, 2kk+1} of row j (colours cA and 1 - cA) in the two planes {i0, i0 + 1}; the i-neighbours
// inside the pair come from the other plane's registers (x(i0 + 1) is plane 1's own x, x(i0)
// plane 0's).  As in k_pass_split the padded arrays let every load be issued unconditionally (a
// plane past the grid reads plane 0's addresses), and selects replace the neighbours outside the
// grid by +0.0.
__device__ __forceinline__ void residual_pair(float* __restrict__ r, int LA, bool hasB, bool ilo, bool ihi, bool jlo,
                                              bool jhi, bool kloA, bool khiB, float xa, float xb, float ba, float bb,
                                              float a_im, float a_ip, float a_jm, float a_jp, float a_km, float b_im,
                                              float b_ip, float b_jm, float b_jp, float b_kp, float h2inv) {
    const float xbv = hasB ? xb : 0.0f;
    {
        float t = 6.0f * xa;
        t = t - (ilo ? a_im : 0.0f);
        t = t - (ihi ? a_ip : 0.0f);
        t = t - (jlo ? a_jm : 0.0f);
        t = t - (jhi ? a_jp : 0.0f);
        t = t - (kloA ? a_km : 0.0f);
        t = t - xbv;
        r[LA] = ba - h2inv * t;
    }
    if (hasB) {
        float t = 6.0f * xbv;
        t = t - (ilo ? b_im : 0.0f);
        t = t - (ihi ? b_ip : 0.0f);
        t = t - (jlo ? b_jm : 0.0f);
        t = t - (jhi ? b_jp : 0.0f);
        t = t - xa;
        t = t - (khiB ? b_kp : 0.0f);
        r[LA + 1] = bb - h2inv * t;
    }
}

// BNAT: b is the natural-layout FP32 right-hand side itself (the finest level of an apply from an FP32
// vector, whose b = RN32(r) = r is then not copied into the split layout); its last element has no
// padding after it, so the second member's load is guarded.
template <bool BNAT = false>
__device__ __forceinline__ void residual_split_body(const float* __restrict__ x, const float* __restrict__ b,
                                                    float* __restrict__ r, Split g, float h2inv, int bx, int by,
                                                    int bz) {
    const int kk = bx * BX + threadIdx.x;
    const int j = by * BY + threadIdx.y;
    const int n = g.n;
    if (j >= n || 2 * kk >= n) return;
    const int i0 = bz * 2;
    const int P = n * n;
    const bool jlo = j > 0, jhi = j + 1 < n, hasB = 2 * kk + 1 < n, kloA = kk > 0, khiB = 2 * kk + 2 < n;
    const bool two = i0 + 1 < n;
    const int LA0 = (i0 * n + j) * n + 2 * kk;
    const int LA1 = two ? LA0 + P : 0;  // a plane past the grid loads harmlessly
    // plane 0
    const int cA0 = (i0 + j) & 1, cB0 = cA0 ^ 1;
    const int mA0 = LA0 >> 1, mB0 = (LA0 + 1) >> 1;
    const float* own0 = x + (cA0 ? g.half : 0);
    const float* oth0 = x + (cA0 ? 0 : g.half);
    const float xa0 = own0[mA0], xb0 = oth0[mA0 + cA0];
    const float ba0 = BNAT ? b[LA0] : b[(cA0 ? g.half : 0) + mA0];
    const float bb0 = BNAT ? (hasB ? b[LA0 + 1] : 0.0f) : b[(cB0 ? g.half : 0) + mB0];
    const float a_im0 = oth0[mA0 + cA0 - g.hP - 1], a_jm0 = oth0[mA0 + cA0 - g.hn - 1], a_jp0 = oth0[mA0 + cA0 + g.hn];
    const float a_km0 = oth0[mA0 + cA0 - 1];
    const float b_im0 = own0[mB0 + cB0 - g.hP - 1], b_jm0 = own0[mB0 + cB0 - g.hn - 1], b_jp0 = own0[mB0 + cB0 + g.hn];
    const float b_kp0 = own0[mB0 + cB0];
    // plane 1 (colours swapped)
    const int cA1 = cB0, cB1 = cA0;
    const int mA1 = LA1 >> 1, mB1 = (LA1 + 1) >> 1;
    const float* own1 = x + (cA1 ? g.half : 0);
    const float* oth1 = x + (cA1 ? 0 : g.half);
    const float xa1 = own1[mA1], xb1 = oth1[mA1 + cA1];
    const float ba1 = BNAT ? b[LA1] : b[(cA1 ? g.half : 0) + mA1];
    const float bb1 = BNAT ? (hasB ? b[LA1 + 1] : 0.0f) : b[(cB1 ? g.half : 0) + mB1];
    const float a_ip1 = oth1[mA1 + cA1 + g.hP], a_jm1 = oth1[mA1 + cA1 - g.hn - 1], a_jp1 = oth1[mA1 + cA1 + g.hn];
    const float a_km1 = oth1[mA1 + cA1 - 1];
    const float b_ip1 = own1[mB1 + cB1 + g.hP], b_jm1 = own1[mB1 + cB1 - g.hn - 1], b_jp1 = own1[mB1 + cB1 + g.hn];
    const float b_kp1 = own1[mB1 + cB1];
    residual_pair(r, LA0, hasB, i0 > 0, two, jlo, jhi, kloA, khiB, xa0, xb0, ba0, bb0, a_im0, xa1, a_jm0, a_jp0, a_km0,
                  b_im0, xb1, b_jm0, b_jp0, b_kp0, h2inv);
    if (two)
        residual_pair(r, LA1, hasB, true, i0 + 2 < n, jlo, jhi, kloA, khiB, xa1, xb1, ba1, bb1, xa0, a_ip1, a_jm1,
                      a_jp1, a_km1, xb0, b_ip1, b_jm1, b_jp1, b_kp1, h2inv);
}

template <bool BNAT = false>
__global__ void __launch_bounds__(BX* BY) k_residual_split(const float* __restrict__ x, const float* __restrict__ b,
                                                            float* __restrict__ r, Split g, float h2inv) {
    pdl_wait();
    pdl_trigger();
    residual_split_body<BNAT>(x, b, r, g, h2inv, blockIdx.x, blockIdx.y, blockIdx.z);
}

// Restriction from a natural-layout fine residual into a split coarse level (odd nc): the
// 27-point sum of k_restrict in the same order, b and b h^2 stored split.  FIRST_X: also the
// coarse level's first smoothing pass (colour 0 from x = 0: x = bs / 6), which the cycle then
// skips.  Split levels come in pairs nf = 2 nc + 1, so all 27 fine points exist: no bounds tests,
// and the 27 loads are issued ahead of the FMA chain.
template <bool FIRST_X>
__device__ __forceinline__ void restrict_split_body(const float* __restrict__ rf, float* __restrict__ bc,
                                                    float* __restrict__ bsc, float* __restrict__ xc, int nf, int nc,
                                                    int halfc, float inv_c, int bx, int by, int bz) {
    // two coarse planes I0 = 2 bz and I0 + 1 a thread: fine plane 2 I0 + 2 serves both (45 loads for two
    // points instead of 54, all issued ahead of the FMA chains), each point summed in k_restrict's order
    const int K = bx * BX + threadIdx.x;
    const int J = by * BY + threadIdx.y;
    const int I0 = 2 * bz;
    if (K >= nc || J >= nc || I0 >= nc) return;
    const bool two = I0 + 1 < nc;
    const float w[3] = {0.25f, 0.5f, 0.25f};
    float v[5][9];  // fine planes 2 I0 .. 2 I0 + 4, rows 2J .. 2J + 2, columns 2K .. 2K + 2
#pragma unroll
    for (int a = 0; a < 5; ++a) {
        if (a >= 3 && !two) break;
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) {
            const float* row = rf + ((2 * I0 + a) * nf + 2 * J + bb) * nf + 2 * K;
#pragma unroll
            for (int c = 0; c < 3; ++c) v[a][bb * 3 + c] = row[c];
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        if (h == 1 && !two) break;
        float acc = 0.0f;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int bb = 0; bb < 3; ++bb) {
                const float wab = w[a] * w[bb];
#pragma unroll
                for (int c = 0; c < 3; ++c) acc = __fmaf_rn(wab * w[c], v[2 * h + a][bb * 3 + c], acc);
            }
        const int Lc = ((I0 + h) * nc + J) * nc + K;
        const int q = split_at(Lc, halfc);
        const float bsv = acc * inv_c;
        bc[q] = acc;
        bsc[q] = bsv;
        if (FIRST_X && !(Lc & 1)) xc[q] = div6(bsv);
    }
}

template <bool FIRST_X>
__global__ void __launch_bounds__(BX* BY) k_restrict_split(const float* __restrict__ rf, float* __restrict__ bc,
                                                           float* __restrict__ bsc, float* __restrict__ xc, int nf,
                                                           int nc, int halfc, float inv_c) {
    pdl_wait();
    pdl_trigger();
    restrict_split_body<FIRST_X>(rf, bc, bsc, xc, nf, nc, halfc, inv_c, blockIdx.x, blockIdx.y, blockIdx.z);
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

// The same correction without the update: returns the weighted sum for fine point (A, B, C) of the cell.
template <int A, int B, int C>
__device__ __forceinline__ float prolong_sum(const float (&X)[2][2][2], const bool (&pi)[2], const bool (&pj)[2],
                                             const bool (&pk)[2]) {
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
    return acc;
}

// Fine x += trilinear interpolation of coarse x (k_prolong's arithmetic) on a split fine level.
// A thread owns the coarse cell (I, J, K), I, J, K in [0, nc], i.e. the fine points
// (2I + a, 2J + b, 2K + c), a, b, c in {0, 1}, inside the grid; it loads the eight coarse values
// around the cell once.  ALL = false: only the colour-0 fine points ((a + b + c) even), the only
// ones the first post-smoothing pass reads.  The coarse level is split (odd nc) or natural.
template <bool SPLIT_C, bool ALL>
__device__ __forceinline__ void prolong_split_body(const float* __restrict__ xc, float* __restrict__ xf, int nc,
                                                   int halfc, int nf, int halff, int bx, int by, int bz) {
    const int K = bx * BX + threadIdx.x;
    const int J = by * BY + threadIdx.y;
    const int I = bz;
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
    if (!ALL) {
        // the four colour-0 points: their fine values are loaded before any is stored (the compiler
        // cannot tell the four addresses apart, and would otherwise wait out each load in turn)
        const int L0 = ((2 * I) * nf + 2 * J) * nf + 2 * K;
        float* e0 = xf + split_at(L0, halff);
        float* e1 = xf + split_at(L0 + nf + 1, halff);       // (0, 1, 1)
        float* e2 = xf + split_at(L0 + nf * nf + 1, halff);  // (1, 0, 1)
        float* e3 = xf + split_at(L0 + nf * nf + nf, halff); // (1, 1, 0)
        const bool h1 = jb && kc, h2 = ia && kc, h3 = ia && jb;
        const float v0 = *e0, v1 = h1 ? *e1 : 0.0f, v2 = h2 ? *e2 : 0.0f, v3 = h3 ? *e3 : 0.0f;
        *e0 = v0 + prolong_sum<0, 0, 0>(X, pi, pj, pk);
        if (h1) *e1 = v1 + prolong_sum<0, 1, 1>(X, pi, pj, pk);
        if (h2) *e2 = v2 + prolong_sum<1, 0, 1>(X, pi, pj, pk);
        if (h3) *e3 = v3 + prolong_sum<1, 1, 0>(X, pi, pj, pk);
        return;
    }
    prolong_point<0, 0, 0>(X, pi, pj, pk, xf, I, J, K, nf, halff);
    if (jb && kc) prolong_point<0, 1, 1>(X, pi, pj, pk, xf, I, J, K, nf, halff);
    if (ia && kc) prolong_point<1, 0, 1>(X, pi, pj, pk, xf, I, J, K, nf, halff);
    if (ia && jb) prolong_point<1, 1, 0>(X, pi, pj, pk, xf, I, J, K, nf, halff);
    {
        if (kc) prolong_point<0, 0, 1>(X, pi, pj, pk, xf, I, J, K, nf, halff);
        if (jb) prolong_point<0, 1, 0>(X, pi, pj, pk, xf, I, J, K, nf, halff);
        if (ia) prolong_point<1, 0, 0>(X, pi, pj, pk, xf, I, J, K, nf, halff);
        if (ia && jb && kc) prolong_point<1, 1, 1>(X, pi, pj, pk, xf, I, J, K, nf, halff);
    }
}

template <bool SPLIT_C, bool ALL>
__global__ void __launch_bounds__(BX* BY) k_prolong_split(const float* __restrict__ xc, float* __restrict__ xf,
                                                          int nc, int halfc, int nf, int halff) {
    pdl_wait();
    pdl_trigger();
    prolong_split_body<SPLIT_C, ALL>(xc, xf, nc, halfc, nf, halff, blockIdx.x, blockIdx.y, blockIdx.z);
}

// b32 = RN32(r), bs32 = RN32(b32 * inv) into the split layout at the finest level; WRITE_X: also
// the cycle's first smoothing pass (colour 0 from x = 0: x = bs / 6).  Thread t handles the
// natural pair L = 2t (colour 0, index t) and L = 2t + 1 (colour 1, index half + t).
// WRITE_B = false: b is not stored (the residual reads the FP32 right-hand side itself, BNAT).
template <bool WRITE_X, class RT, bool WRITE_B = true>
__global__ void k_scale_in32_split(const RT* __restrict__ r, float* __restrict__ b, float* __restrict__ bs,
                                   float* __restrict__ x, float inv, int N, int half) {
    pdl_wait();
    pdl_trigger();
    const int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < half; t += stride) {
        const int L = 2 * t;
        const float v0 = f64_to_f32(r[L]);
        const float s0 = v0 * inv;
        if (WRITE_B) b[t] = v0;
        bs[t] = s0;
        if (WRITE_X) x[t] = div6(s0);
        if (L + 1 < N) {
            const float v1 = f64_to_f32(r[L + 1]);
            if (WRITE_B) b[half + t] = v1;
            bs[half + t] = v1 * inv;
        }
    }
}

// cc = the full-weighting restriction of a natural-layout coefficient (weights (1/4, 1/2, 1/4) per
// dimension, summed z outer, y, x inner), FP32 out.  An FP64 input is rounded to FP32 by the integer
// conversion (the hardware one issues on the FP64 pipe).  A thread owns a coarse (K, J) column and
// marches I: fine plane 2I+2 of one step is plane 2I of the next, kept in registers, so a coarse point
// loads 18 fine values, not 27.
template <class TI>
__device__ __forceinline__ void restrict_coef_body(const TI* __restrict__ cf, float* __restrict__ cc, int nf, int nc,
                                                   int ichunk, int bx, int by, int bz) {
    const int K = bx * BX + threadIdx.x;
    const int J = by * BY + threadIdx.y;
    if (K >= nc || J >= nc) return;
    const int I0 = bz * ichunk;
    const int I1 = min(I0 + ichunk, nc);
    const float w[3] = {0.25f, 0.5f, 0.25f};
    const size_t pf = (size_t)nf * nf;
    const size_t col = (size_t)(2 * J) * nf + 2 * K;  // fine (2J, 2K) within a plane
    auto load_plane = [&](int i, float (&v)[9]) {
        const TI* q = cf + (size_t)i * pf + col;
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
            for (int c = 0; c < 3; ++c) v[b * 3 + c] = f64_to_f32(q[(size_t)b * nf + c]);
    };
    float p0[9], p1[9], p2[9];
    load_plane(2 * I0, p0);
    for (int I = I0; I < I1; ++I) {
        load_plane(2 * I + 1, p1);
        load_plane(2 * I + 2, p2);
        float acc = 0.0f;
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
            for (int c = 0; c < 3; ++c) acc = __fmaf_rn(w[0] * w[b] * w[c], p0[b * 3 + c], acc);
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
            for (int c = 0; c < 3; ++c) acc = __fmaf_rn(w[1] * w[b] * w[c], p1[b * 3 + c], acc);
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
            for (int c = 0; c < 3; ++c) acc = __fmaf_rn(w[2] * w[b] * w[c], p2[b * 3 + c], acc);
        cc[((size_t)I * nc + J) * nc + K] = acc;
#pragma unroll
        for (int q = 0; q < 9; ++q) p0[q] = p2[q];
    }
}

// z (FP64, natural) = x (FP32, split)
__global__ void k_to64_split(const float* __restrict__ x, double* __restrict__ z, int N, int half) {
    pdl_wait();
    pdl_trigger();
    const int stride = gridDim.x * blockDim.x;
    for (int L = blockIdx.x * blockDim.x + threadIdx.x; L < N; L += stride) z[L] = f32_to_f64(x[split_at(L, half)]);
}

// ------------------------------------------------------------------------------------------
// The tail of a V-cycle in one CTA: every level from lb (n <= 15) down to the coarsest, with all
// arrays in shared memory (natural layout) and __syncthreads() between passes instead of one
// kernel launch per pass.  The arithmetic of each step is that of the per-level kernels above
// (colour pass, residual, restriction, prolongation, single-point solve), so the result is the
// same as the launched sequence.  Level lb's b and b h^2 come from global memory (split layout
// when SPLIT_IO) and its x goes back there for the prolongation into the level above.
constexpr int kMaxTail = 6;
struct TailParams {
    int levels;                  // levels handled: lb .. lb + levels - 1 (the coarsest)
    int n[kMaxTail];
    double h2inv[kMaxTail];      // h^-2 of each level
    double inv[kMaxTail];        // 1 / h^-2 of each level (b h^2 = b * inv)
    double six_h2inv[kMaxTail];  // 6 h^-2 (single-point solve)
    int pre, post;
    int half;                    // split geometry of level lb (SPLIT_IO)
    // Jacobian-aware coarse levels (FP32 only): c[l] = the coefficient c of -Lap_h - c on level l
    // (natural layout, global memory), or null everywhere for the Poisson tail.
    const float* c[kMaxTail];
};

// NC > 0: the level's n as a compile-time constant (the index divisions become multiplications);
// 0: the runtime n_rt.
// cs (may be null): c h^2 per point: the pass then solves for -Lap_h - c, x = (b h^2 + sum) / (6 - c h^2).
template <class T, int NC>
__device__ void tail_pass(T* __restrict__ x, const T* __restrict__ bs, int n_rt, int c, bool first,
                          const T* __restrict__ cs = nullptr) {
    const int n = NC ? NC : n_rt;
    const int np = (n + 1) / 2, total = n * n * np, P = n * n;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int kk = t % np, row = t / np, j = row % n, i = row / n;
        const int k = 2 * kk + ((i + j + c) & 1);
        if (k >= n) continue;
        const int p = (i * n + j) * n + k;
        T acc = bs[p];
        if (!first) {
            acc = acc + ((i > 0) ? x[p - P] : zero<T>());
            acc = acc + ((i + 1 < n) ? x[p + P] : zero<T>());
            acc = acc + ((j > 0) ? x[p - n] : zero<T>());
            acc = acc + ((j + 1 < n) ? x[p + n] : zero<T>());
            acc = acc + ((k > 0) ? x[p - 1] : zero<T>());
            acc = acc + ((k + 1 < n) ? x[p + 1] : zero<T>());
        }
        x[p] = cs ? acc / (T(6) - cs[p]) : div6(acc);
    }
    __syncthreads();
}

// cs (may be null): c h^2 per point: r = b - h^-2 (6x - sum - c h^2 x), the residual of -Lap_h - c.
template <class T, int NC>
__device__ void tail_residual(const T* __restrict__ x, const T* __restrict__ b, T* __restrict__ r, int n_rt,
                              T h2inv, const T* __restrict__ cs = nullptr) {
    const int n = NC ? NC : n_rt;
    const int N = n * n * n, P = n * n;
    for (int p = threadIdx.x; p < N; p += blockDim.x) {
        const int k = p % n, j = (p / n) % n, i = p / P;
        T s = T(6) * x[p];
        s = s - ((i > 0) ? x[p - P] : zero<T>());
        s = s - ((i + 1 < n) ? x[p + P] : zero<T>());
        s = s - ((j > 0) ? x[p - n] : zero<T>());
        s = s - ((j + 1 < n) ? x[p + n] : zero<T>());
        s = s - ((k > 0) ? x[p - 1] : zero<T>());
        s = s - ((k + 1 < n) ? x[p + 1] : zero<T>());
        if (cs) s = s - cs[p] * x[p];
        r[p] = b[p] - h2inv * s;
    }
    __syncthreads();
}

template <class T, int NF>  // NF > 0: nf = NF and nc = (NF - 1) / 2 at compile time
__device__ void tail_restrict(const T* __restrict__ rf, T* __restrict__ bc, T* __restrict__ bsc, int nf_rt,
                              int nc_rt, T inv_c) {
    const int nf = NF ? NF : nf_rt, nc = NF ? (NF - 1) / 2 : nc_rt;
    const int Nc = nc * nc * nc;
    const T w[3] = {T(0.25), T(0.5), T(0.25)};
    for (int q = threadIdx.x; q < Nc; q += blockDim.x) {
        const int K = q % nc, J = (q / nc) % nc, I = q / (nc * nc);
        T acc = zero<T>();
        for (int a = 0; a < 3; ++a) {
            const int fi = 2 * I + a;
            if (fi >= nf) continue;
            for (int bb = 0; bb < 3; ++bb) {
                const int fj = 2 * J + bb;
                if (fj >= nf) continue;
                const T wab = w[a] * w[bb];
                for (int c = 0; c < 3; ++c) {
                    const int fk = 2 * K + c;
                    if (fk >= nf) continue;
                    acc = fma_t(wab * w[c], rf[(fi * nf + fj) * nf + fk], acc);
                }
            }
        }
        bc[q] = acc;
        bsc[q] = acc * inv_c;
    }
    __syncthreads();
}

template <class T, int NF>  // NF > 0: nf = NF and nc = (NF - 1) / 2 at compile time
__device__ void tail_prolong(const T* __restrict__ xc, T* __restrict__ xf, int nc_rt, int nf_rt, bool colour0_only) {
    const int nf = NF ? NF : nf_rt, nc = NF ? (NF - 1) / 2 : nc_rt;
    const int Nf = nf * nf * nf;
    for (int p = threadIdx.x; p < Nf; p += blockDim.x) {
        const int k = p % nf, j = (p / nf) % nf, i = p / (nf * nf);
        if (colour0_only && ((i + j + k) & 1)) continue;
        int ci[2], cj[2], ck[2];
        const int ni = interp(i, nc, ci), nj = interp(j, nc, cj), nk = interp(k, nc, ck);
        const T wi = (ni == 1 && (i & 1)) ? T(1) : T(0.5);
        const T wj = (nj == 1 && (j & 1)) ? T(1) : T(0.5);
        const T wk = (nk == 1 && (k & 1)) ? T(1) : T(0.5);
        T acc = zero<T>();
        for (int a = 0; a < ni; ++a)
            for (int bb = 0; bb < nj; ++bb)
                for (int c = 0; c < nk; ++c) acc = fma_t(wi * wj * wk, xc[(ci[a] * nc + cj[bb]) * nc + ck[c]], acc);
        xf[p] = xf[p] + acc;
    }
    __syncthreads();
}

// Calls f with n as a compile-time constant for the tail's usual sizes (odd chains 15, 7, 3), else
// with 0 (runtime n).  A constant is used only where the next level is (n - 1) / 2.
template <class F>
__device__ __forceinline__ void with_tail_n(int n, int n_next, F&& f) {
    const bool chain = n_next == (n - 1) / 2;
    if (n == 15 && chain) f(std::integral_constant<int, 15>{});
    else if (n == 7 && chain) f(std::integral_constant<int, 7>{});
    else if (n == 3 && chain) f(std::integral_constant<int, 3>{});
    else f(std::integral_constant<int, 0>{});
}

template <class T, bool SPLIT_IO>
__device__ __forceinline__ void mg_tail_body(const T* __restrict__ b_g, const T* __restrict__ bs_g,
                                             T* __restrict__ x_g, const TailParams& tp) {
    extern __shared__ __align__(16) unsigned char tail_smem[];
    T* base = reinterpret_cast<T*>(tail_smem);
    T *X[kMaxTail], *B[kMaxTail], *BS[kMaxTail], *CS[kMaxTail];
    const bool shift = tp.c[0] != nullptr;
    int off = 0;
    for (int l = 0; l < tp.levels; ++l) {
        const int Nl = tp.n[l] * tp.n[l] * tp.n[l];
        X[l] = base + off;
        B[l] = base + off + Nl;
        BS[l] = base + off + 2 * Nl;
        off += 3 * Nl;
    }
    T* R = base + off;  // residual scratch, the size of level lb
    off += tp.n[0] * tp.n[0] * tp.n[0];
    for (int l = 0; l < tp.levels; ++l) {
        CS[l] = nullptr;
        if (!shift) continue;
        // c h^2 of the level (the shift in the units of b h^2)
        const int Nl = tp.n[l] * tp.n[l] * tp.n[l];
        CS[l] = base + off;
        off += Nl;
        const T inv = (T)tp.inv[l];
        for (int p = threadIdx.x; p < Nl; p += blockDim.x) CS[l][p] = (T)tp.c[l][p] * inv;
    }
    {
        const int n = tp.n[0], N = n * n * n;
        for (int p = threadIdx.x; p < N; p += blockDim.x) {
            const int q = SPLIT_IO ? split_at(p, tp.half) : p;
            B[0][p] = b_g[q];
            BS[0][p] = bs_g[q];
        }
        __syncthreads();
    }
    const int last = tp.levels - 1;
    for (int l = 0; l < last; ++l) {  // down: pre-smoothing, residual, restriction
        const int n = tp.n[l];
        with_tail_n(n, tp.n[l + 1], [&](auto nc) {
            constexpr int NC = decltype(nc)::value;
            for (int sw = 0; sw < tp.pre; ++sw) {
                tail_pass<T, NC>(X[l], BS[l], n, 0, sw == 0, CS[l]);
                tail_pass<T, NC>(X[l], BS[l], n, 1, false, CS[l]);
            }
            if (tp.pre == 0) {
                for (int p = threadIdx.x; p < n * n * n; p += blockDim.x) X[l][p] = zero<T>();
                __syncthreads();
            }
            tail_residual<T, NC>(X[l], B[l], R, n, (T)tp.h2inv[l], CS[l]);
            tail_restrict<T, NC>(R, B[l + 1], BS[l + 1], n, tp.n[l + 1], (T)tp.inv[l + 1]);
        });
    }
    {  // coarsest
        const int n = tp.n[last];
        if (n == 1) {
            if (threadIdx.x == 0) {
                if (shift) X[last][0] = B[last][0] / ((T)tp.six_h2inv[last] - (T)tp.c[last][0]);
                else X[last][0] = (T)((double)B[last][0] / tp.six_h2inv[last]);
            }
            __syncthreads();
        } else {
            for (int sw = 0; sw < 30; ++sw) {
                const int c0 = (sw % 2 == 0) ? 0 : 1;
                tail_pass<T, 0>(X[last], BS[last], n, c0, sw == 0, CS[last]);
                tail_pass<T, 0>(X[last], BS[last], n, 1 - c0, false, CS[last]);
            }
        }
    }
    for (int l = last - 1; l >= 0; --l) {  // up: prolongation, post-smoothing
        const int n = tp.n[l];
        with_tail_n(n, tp.n[l + 1], [&](auto nc) {
            constexpr int NC = decltype(nc)::value;
            tail_prolong<T, NC>(X[l + 1], X[l], tp.n[l + 1], n, tp.post > 0);
            for (int sw = 0; sw < tp.post; ++sw) {
                tail_pass<T, NC>(X[l], BS[l], n, 1, false, CS[l]);
                tail_pass<T, NC>(X[l], BS[l], n, 0, false, CS[l]);
            }
        });
    }
    {
        const int n = tp.n[0], N = n * n * n;
        for (int p = threadIdx.x; p < N; p += blockDim.x) x_g[SPLIT_IO ? split_at(p, tp.half) : p] = X[0][p];
    }
}

template <class T, bool SPLIT_IO>
__global__ void __launch_bounds__(1024) k_mg_tail(const T* __restrict__ b_g, const T* __restrict__ bs_g,
                                                 T* __restrict__ x_g, TailParams tp) {
    pdl_wait();
    pdl_trigger();
    mg_tail_body<T, SPLIT_IO>(b_g, bs_g, x_g, tp);
}

}  // namespace
}  // namespace numa::gpu
