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
// A block owns a 32 (k) x 16 (j) tile and a chunk of i planes and streams the planes through
// shared memory: x planes with a 2-point halo in a ring of five slots, b h^2 planes with a
// 1-point halo in a ring of three.  Step p: start the asynchronous copies (cp.async) of x plane
// p+2 and b h^2 plane p+1; wait for those of the step before; update colour c0 of plane p over
// the tile plus a 1-point halo (its in-plane neighbours reach 2 points out); update colour c1
// of plane p-1 over the tile (all its neighbours are final colour-c0 values); store plane p-1.
// The copies of one step overlap the arithmetic of the previous one.
// The sweep is out of place (xin -> xout): blocks read halo planes that neighbouring blocks
// write, so reads must see the values from before the sweep.  FIRST: xin is zero (no loads).
constexpr int SW_TK = 32, SW_TJ = 16;
constexpr int SW_SK = SW_TK + 4, SW_SJ = SW_TJ + 4;  // x tile with a 2-point halo
constexpr int SW_BK = SW_TK + 2, SW_BJ = SW_TJ + 2;  // b h^2 tile with a 1-point halo
constexpr int SW_PLANE = SW_SK * SW_SJ;
constexpr int SW_BPLANE = SW_BK * SW_BJ;
constexpr int SW_THREADS = 256;
constexpr int SW_XSLOTS = 5, SW_BSLOTS = 3;

__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    const int n = valid ? 4 : 0;  // 0: nothing is read, the 4 bytes are zero-filled
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
}

// Every thread's roles are fixed for the whole kernel and their offsets computed once: three
// elements of each x-plane copy and of each b h^2-plane copy, two horizontally adjacent halo
// positions for the colour-c0 update (exactly one of the two has colour c0 on any plane), two
// adjacent interior positions for the colour-c1 update, two interior values to store.
template <bool FIRST, bool OUT_X, bool OUT_Z>
__global__ void __launch_bounds__(SW_THREADS) k_rbgs_sweep32(const float* __restrict__ xin, float* __restrict__ xout,
                                                            const float* __restrict__ bs, double* __restrict__ z,
                                                            int n, int c0, int ichunk) {
    __shared__ float X[SW_XSLOTS * SW_PLANE];
    __shared__ float B[SW_BSLOTS * SW_BPLANE];
    const int tid = threadIdx.x;
    const int k0 = blockIdx.x * SW_TK, j0 = blockIdx.y * SW_TJ;
    const int ib = blockIdx.z * ichunk;
    const int ie = min(ib + ichunk, n);
    const size_t plane = (size_t)n * n;

    // copies: element e of the x tile (row e / SW_SK) and of the b h^2 tile (row e / SW_BK)
    int xg[3], bg[3];
    bool xv[3], bv[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int e = tid + q * SW_THREADS;
        int r = e / SW_SK, c = e - r * SW_SK;
        int j = j0 - 2 + r, k = k0 - 2 + c;
        xv[q] = e < SW_PLANE && j >= 0 && j < n && k >= 0 && k < n;
        xg[q] = xv[q] ? j * n + k : 0;
        r = e / SW_BK;
        c = e - r * SW_BK;
        j = j0 - 1 + r;
        k = k0 - 1 + c;
        bv[q] = e < SW_BPLANE && j >= 0 && j < n && k >= 0 && k < n;
        bg[q] = bv[q] ? j * n + k : 0;
    }
    // colour-c0 pairs over the 1-point halo: 18 rows x 17 pairs (k0-1+2q, k0+2q)
    constexpr int NPAIR0 = (SW_TJ + 2) * ((SW_TK + 2) / 2);
    int h_xo[2], h_bo[2], h_par[2];
    bool h_va[2], h_vb[2], h_on[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int t = tid + q * SW_THREADS;
        h_on[q] = t < NPAIR0;
        const int r = t / ((SW_TK + 2) / 2), qq = t - r * ((SW_TK + 2) / 2);
        const int j = j0 - 1 + r, ka = k0 - 1 + 2 * qq;
        h_xo[q] = (r + 1) * SW_SK + (2 * qq + 1);
        h_bo[q] = r * SW_BK + 2 * qq;
        h_par[q] = (j + ka) & 1;
        const bool jin = j >= 0 && j < n;
        h_va[q] = h_on[q] && jin && ka >= 0 && ka < n;
        h_vb[q] = h_on[q] && jin && ka + 1 < n;
    }
    // colour-c1 pair in the interior: row tid / 16, columns k0+2q, k0+2q+1
    const int ir = tid / (SW_TK / 2), iq = tid - ir * (SW_TK / 2);
    const int i_xo = (ir + 2) * SW_SK + (2 * iq + 2);
    const int i_bo = (ir + 1) * SW_BK + (2 * iq + 1);
    const int i_par = (j0 + ir + k0 + 2 * iq) & 1;
    const bool i_va = j0 + ir < n && k0 + 2 * iq < n;
    const bool i_vb = j0 + ir < n && k0 + 2 * iq + 1 < n;
    // stores: interior elements tid and tid + 256 (row e / 32)
    int s_xo[2], s_g[2];
    bool s_v[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int e = tid + q * SW_THREADS;
        const int r = e / SW_TK, c = e - r * SW_TK;
        s_xo[q] = (r + 2) * SW_SK + (c + 2);
        s_v[q] = j0 + r < n && k0 + c < n;
        s_g[q] = s_v[q] ? (j0 + r) * n + (k0 + c) : 0;
    }

    auto load_x = [&](int p, float* S) {
        const bool pin = p >= 0 && p < n;
        const float* src = xin + (pin ? (size_t)p * plane : 0);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const int e = tid + q * SW_THREADS;
            if (e < SW_PLANE) {
                if (FIRST) S[e] = 0.0f;
                else cp_async4(S + e, src + xg[q], pin && xv[q]);
            }
        }
    };
    auto load_b = [&](int p, float* S) {
        const bool pin = p >= 0 && p < n;
        const float* src = bs + (pin ? (size_t)p * plane : 0);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const int e = tid + q * SW_THREADS;
            if (e < SW_BPLANE) cp_async4(S + e, src + bg[q], pin && bv[q]);
        }
    };
    auto gs = [](const float* Bp, const float* Xm, float* X0, const float* Xp, int xo, int bo) {
        float acc = Bp[bo];
        acc = acc + Xm[xo];
        acc = acc + Xp[xo];
        acc = acc + X0[xo - SW_SK];
        acc = acc + X0[xo + SW_SK];
        acc = acc + X0[xo - 1];
        acc = acc + X0[xo + 1];
        X0[xo] = div6(acc);
    };
    // colour c0 of plane p (ring slots of p-1, p, p+1 and its b h^2 slot)
    auto upd0 = [&](int p, const float* Xm, float* X0, const float* Xp, const float* Bp) {
        if (p < 0 || p >= n) return;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (!h_on[q]) continue;
            const bool first = ((p + h_par[q]) & 1) == c0;  // the even-column member has colour c0
            if (first ? h_va[q] : h_vb[q]) gs(Bp, Xm, X0, Xp, h_xo[q] + (first ? 0 : 1), h_bo[q] + (first ? 0 : 1));
        }
    };
    auto upd1 = [&](int p, const float* Xm, float* X0, const float* Xp, const float* Bp) {
        const bool first = ((p + i_par) & 1) != c0;  // colour c1 = the other colour
        if (first ? i_va : i_vb) gs(Bp, Xm, X0, Xp, i_xo + (first ? 0 : 1), i_bo + (first ? 0 : 1));
    };
    auto store = [&](int p, const float* S) {
        const size_t base = (size_t)p * plane;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (!s_v[q]) continue;
            const float v = S[s_xo[q]];
            if (OUT_X) xout[base + s_g[q]] = v;
            if (OUT_Z) z[base + s_g[q]] = f32_to_f64(v);
        }
    };
    auto xslot = [&](int s) { return X + s * SW_PLANE; };
    auto bslot = [&](int s) { return B + s * SW_BPLANE; };
    auto wrap5 = [](int s) { return s >= SW_XSLOTS ? s - SW_XSLOTS : s; };
    auto wrap3 = [](int s) { return s >= SW_BSLOTS ? s - SW_BSLOTS : s; };

    // ring positions: x plane q lives in slot (q - ib + 2) mod 5, b h^2 plane q in (q - ib + 1) mod 3
    load_x(ib - 2, xslot(0));
    load_x(ib - 1, xslot(1));
    load_x(ib, xslot(2));
    load_x(ib + 1, xslot(3));
    load_b(ib - 1, bslot(0));
    load_b(ib, bslot(1));
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    upd0(ib - 1, xslot(0), xslot(1), xslot(2), bslot(0));
    int sx = 2, sb = 1;  // slots of x plane p and b h^2 plane p
    for (int p = ib; p <= ie; ++p) {
        __syncthreads();
        load_x(p + 2, xslot(wrap5(sx + 2)));
        load_b(p + 1, bslot(wrap3(sb + 1)));
        cp_async_commit();
        cp_async_wait<1>();
        __syncthreads();
        float* Xm1 = xslot(wrap5(sx + 4));
        float* X0 = xslot(sx);
        upd0(p, Xm1, X0, xslot(wrap5(sx + 1)), bslot(sb));
        __syncthreads();
        if (p - 1 >= ib) {
            upd1(p - 1, xslot(wrap5(sx + 3)), Xm1, X0, bslot(wrap3(sb + 2)));
            __syncthreads();
            store(p - 1, Xm1);
        }
        sx = wrap5(sx + 1);
        sb = wrap3(sb + 1);
    }
    cp_async_wait<0>();
}

}  // namespace
}  // namespace numa::gpu
