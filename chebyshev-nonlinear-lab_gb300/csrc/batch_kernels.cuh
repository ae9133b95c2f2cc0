// batch_kernels.cuh — kernels of the batched Bratu3D solver (batch_solver.cu): many instances of
// uneven grid size advanced together, one launch per operation over all of them.
//
// Packed instance table.  Instances are ordered by grid size (largest first), and every grid
// vector of the batch (iterate, residual, Krylov basis ...) is one packed array of T = sum n_i^3
// values in which instance t occupies [off_t, off_t + n_t^3).  Instances of one size form a class
// and sit next to each other, so a class is a uniform run of same-shaped grids: a stencil launch
// covers a whole class with blockIdx.z = grid * (plane chunks) + chunk.  Element-wise passes run
// over a block table (block -> instance and element range) that covers every instance, and their
// per-block partial sums are reduced per instance in block order (deterministic).
//
// Multigrid pools.  The V-cycle runs over pools of same-shaped levels: pool s holds the level of
// size s of every instance with n >= s (the largest instances first), so one launch smooths,
// restricts or prolongs that level for the whole batch, and the coarse levels of all instances
// run side by side instead of one short kernel each.  Pool grid q of size s and pool grid q of
// size 2s + 1 belong to the same instance.  The instances whose finest level is s are the last
// grids of pool s.
//
// Every kernel checks its instance's activity flag first: an instance that has converged, or whose
// linear solve has ended, costs its blocks an early exit.
#pragma once

#include "mg_kernels.cuh"

namespace numa::gpu {
namespace {

// ------------------------------------------------------------------------------ the pools
// One pool of same-shaped split levels: grid q keeps x at x + q sx (past its front padding), b and
// b h^2 at b + q sb and bs + q sb, its natural-layout residual at r + q sr; inst[q] = its instance.
struct MgPool {
    float* x;
    float* b;
    float* bs;
    float* r;
    long long sx, sb, sr;
    const int* inst;
};

__device__ __forceinline__ bool pool_active(const MgPool& P, const int* act, int q) {
    return act == nullptr || act[P.inst[q]] != 0;
}

// b, b h^2 of the pool grids g0 .. g0 + gridDim.y - 1 from their instances' FP32 right-hand side
// (rhs + (q - g0) rs: a class of the packed basis), WRITE_X: with the first colour-0 pass.
template <bool WRITE_X>
__global__ void k_bscale_in(const float* __restrict__ rhs, long long rs, MgPool P, const int* __restrict__ act, int g0,
                            float inv, int N, int half) {
    pdl_wait();
    pdl_trigger();
    const int q = g0 + blockIdx.y;
    if (!pool_active(P, act, q)) return;
    const float* r = rhs + (long long)blockIdx.y * rs;
    float* b = P.b + q * P.sb;
    float* bs = P.bs + q * P.sb;
    float* x = P.x + q * P.sx;
    const int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < half; t += stride) {
        const int L = 2 * t;
        const float v0 = r[L];
        const float s0 = v0 * inv;
        b[t] = v0;
        bs[t] = s0;
        if (WRITE_X) x[t] = div6(s0);
        if (L + 1 < N) {
            const float v1 = r[L + 1];
            b[half + t] = v1;
            bs[half + t] = v1 * inv;
        }
    }
}

// One colour pass over pool grids g0 .. (zch blocks of z per grid).  kPassLastZ: z32 of grid q at
// z32 + (q - g0) zs (the instance's preconditioned Krylov vector).
template <int MODE, int ICH, int NN>
__global__ void __launch_bounds__(BX* BY) k_bpass(MgPool P, const int* __restrict__ act, int g0, int zch, Split g,
                                                  int c, float* __restrict__ z32, long long zs) {
    pdl_wait();
    pdl_trigger();
    const int gq = blockIdx.z / zch, q = g0 + gq;
    if (!pool_active(P, act, q)) return;
    float* x = P.x + q * P.sx;
    float* own = x + (c ? g.half : 0);
    const float* oth = x + (c ? 0 : g.half);
    const float* bown = P.bs + q * P.sb + (c ? g.half : 0);
    float* zq = z32 ? z32 + (long long)gq * zs : nullptr;
    pass_split_body<MODE, ICH, NN>(own, oth, bown, nullptr, g, c, zq, blockIdx.x, blockIdx.y, blockIdx.z - gq * zch);
}

__global__ void __launch_bounds__(BX* BY) k_bresidual(MgPool P, const int* __restrict__ act, int zch, Split g,
                                                      float h2inv) {
    pdl_wait();
    pdl_trigger();
    const int q = blockIdx.z / zch;
    if (!pool_active(P, act, q)) return;
    residual_split_body<false>(P.x + q * P.sx, P.b + q * P.sb, P.r + q * P.sr, g, h2inv, blockIdx.x, blockIdx.y,
                        blockIdx.z - q * zch);
}

// fine pool grid q -> coarse pool grid q (the same instance), (nc + 1) / 2 plane pairs per grid
template <bool FIRST_X>
__global__ void __launch_bounds__(BX* BY) k_brestrict(MgPool F, MgPool C, const int* __restrict__ act, int nf, int nc,
                                                      int halfc, float inv_c) {
    pdl_wait();
    pdl_trigger();
    const int zc = (nc + 1) / 2;  // two coarse planes a thread
    const int q = blockIdx.z / zc;
    if (!pool_active(F, act, q)) return;
    restrict_split_body<FIRST_X>(F.r + q * F.sr, C.b + q * C.sb, C.bs + q * C.sb, C.x + q * C.sx, nf, nc, halfc, inv_c,
                                 blockIdx.x, blockIdx.y, blockIdx.z - q * zc);
}

// coarse pool grid q -> fine pool grid q, nc + 1 cell planes per grid
template <bool ALL>
__global__ void __launch_bounds__(BX* BY) k_bprolong(MgPool C, MgPool F, const int* __restrict__ act, int nc, int halfc,
                                                     int nf, int halff) {
    pdl_wait();
    pdl_trigger();
    const int q = blockIdx.z / (nc + 1);
    if (!pool_active(F, act, q)) return;
    prolong_split_body<true, ALL>(C.x + q * C.sx, F.x + q * F.sx, nc, halfc, nf, halff, blockIdx.x, blockIdx.y,
                                  blockIdx.z - q * (nc + 1));
}

// the levels n <= 15 of every pool grid: one CTA per grid.  With tp.c set (Jacobian-aware tail), level m's
// coefficients of grid q are at tp.c[m] + q n_m^3.
__global__ void __launch_bounds__(1024) k_btail(MgPool P, const int* __restrict__ act, TailParams tp) {
    pdl_wait();
    pdl_trigger();
    const int q = blockIdx.x;
    if (!pool_active(P, act, q)) return;
    if (tp.c[0])
        for (int m = 0; m < tp.levels; ++m) tp.c[m] += (size_t)q * tp.n[m] * tp.n[m] * tp.n[m];
    mg_tail_body<float, true>(P.b + q * P.sb, P.bs + q * P.sb, P.x + q * P.sx, tp);
}

// The Jacobian coefficient of grids g0 .. of a coarse level: the full-weighting restriction of the
// finer level's (natural layout, grid q of the source at src + (q - g0) ss), into dst + q sd; zch plane
// chunks of ichunk coarse planes a grid.  The arithmetic of the single-instance hierarchy's.
__global__ void __launch_bounds__(BX* BY) k_brestrict_coef(const float* __restrict__ src, long long ss,
                                                           float* __restrict__ dst, long long sd,
                                                           const int* __restrict__ inst, const int* __restrict__ act,
                                                           int g0, int nf, int nc, int ichunk, int zch) {
    pdl_wait();
    pdl_trigger();
    const int gq = blockIdx.z / zch, q = g0 + gq;
    if (act && !act[inst[q]]) return;
    restrict_coef_body(src + (long long)gq * ss, dst + (long long)q * sd, nf, nc, ichunk, blockIdx.x, blockIdx.y,
                       blockIdx.z - gq * zch);
}

// ------------------------------------------------------------------------------ stencils
constexpr int kBX = 32, kBY = 8;

// One class of instances: grids t0 .. t0 + count - 1 of size n, packed at off0 + (t - t0) N.
struct BClass {
    int n, t0, kb, jb, zch, ichunk;
    long long N, off0;
    float h2inv32;
    double h2inv;
    int pbase;  // first partial slot of the class (stencil reductions)
};

// The exp table scaled by each instance's lambda (the single-instance operator's k_lam_table, one table of
// 2^kExpTableBits entries an instance, blockIdx.y = instance - t0): T2 = (RN(lambda T_hi), lambda T_hi -
// RN(lambda T_hi) + lambda T_lo), TF their RN32.  Instances with lambda outside [2^-10, 2^10] keep no table.
__global__ void k_blam_tables(const double* __restrict__ lam, double2* __restrict__ T2, float2* __restrict__ TF,
                              int t0) {
    const int t = t0 + blockIdx.y;
    const int jj = blockIdx.x * blockDim.x + threadIdx.x;
    if (jj >= (1 << kExpTableBits)) return;
    const double l = lam[t];
    const double2 T = kExp2Frac[jj];
    const double hi = __dmul_rn(l, T.x);
    const double lo = __dadd_rn(__fma_rn(l, T.x, -hi), __dmul_rn(l, T.y));
    T2[(size_t)t * (1 << kExpTableBits) + jj] = make_double2(hi, lo);
    TF[(size_t)t * (1 << kExpTableBits) + jj] = make_float2(__double2float_rn(hi), __double2float_rn(lo));
}

// F = h^-2 (6 u - sum) - lambda e^u at the instances with eval[t] set, from x_a or x_b (the one
// selected by cur[t] ^ which), with RN32(lambda e^u) into c32, RN32(F) into f32 (the first FP32
// Krylov vector of the next linear solve) and the block's sum of F^2 into partials: the arithmetic
// of the single-instance residual kernel (its fixed-point 7-point sum, lambda e^u from a lambda-scaled
// exp table per instance).  Held to five resident CTAs an SM (48 registers), as the
// single-instance kernel: its integer and FP64 pipes are both busy, and the extra warps cover latency.
__global__ void __launch_bounds__(kBX* kBY, 5) k_beval(const double* __restrict__ xa, const double* __restrict__ xb,
                                                    const int* __restrict__ cur, int which,
                                                    const int* __restrict__ eval, const double* __restrict__ lam,
                                                    BClass C, double* __restrict__ F, float* __restrict__ c32,
                                                    float* __restrict__ f32, double* __restrict__ partials,
                                                    const double2* __restrict__ lt2, const float2* __restrict__ ltf) {
    pdl_wait();
    pdl_trigger();
    const int gq = blockIdx.z / C.zch, bz = blockIdx.z - gq * C.zch;
    const int t = C.t0 + gq;
    if (!eval[t]) return;
    const int n = C.n;
    const long long base = C.off0 + (long long)gq * C.N;
    const double* u = ((cur[t] ^ which) ? xb : xa) + base;
    const double lm = lam[t], h2inv = C.h2inv;
    // lambda e^u from the instance's lambda-scaled table (one FP64 multiply fewer), as the single-instance
    // operator does for lambda in [2^-10, 2^10]
    const bool lt_on = lm >= 0x1p-10 && lm <= 0x1p10;
    const double2* T2 = lt2 + (size_t)t * (1 << kExpTableBits);
    const float2* TF = ltf + (size_t)t * (1 << kExpTableBits);
    const int k = blockIdx.x * kBX + threadIdx.x;
    const int j = blockIdx.y * kBY + threadIdx.y;
    const int i0 = bz * C.ichunk;
    const int i1 = min(i0 + C.ichunk, n);
    const size_t plane = (size_t)n * n;
    double acc[1] = {0.0};
    if (k < n && j < n) {
        size_t p = ((size_t)i0 * n + j) * n + k;
        double below = (i0 > 0) ? u[p - plane] : 0.0;
        double curv = u[p];
        for (int i = i0; i < i1; ++i) {
            const double above = (i + 1 < n) ? u[p + plane] : 0.0;
            const double jm = (j > 0) ? u[p - n] : 0.0;
            const double jp = (j + 1 < n) ? u[p + n] : 0.0;
            const double km = (k > 0) ? u[p - 1] : 0.0;
            const double kp = (k + 1 < n) ? u[p + 1] : 0.0;
            // as the single-instance mixed evaluation: the 7-point sum in 64-bit fixed point, rounded once
            const double s = lap7_fixed(curv, below, above, jm, jp, km, kp);
            const double e = lt_on ? lam_exp_tang(curv, lm, T2, TF) : lm * exp_tang(curv);
            const double f = __fma_rn(h2inv, s, -e);
            F[base + p] = f;
            c32[base + p] = f64_to_f32(e);
            f32[base + p] = f64_to_f32(f);
            acc[0] = __fma_rn(f, f, acc[0]);
            below = curv;
            curv = above;
            p += plane;
        }
    }
    __shared__ double sm[1][32];
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0 && threadIdx.y == 0)
        partials[C.pbase + ((size_t)(gq * C.zch + bz) * C.jb + blockIdx.y) * C.kb + blockIdx.x] = acc[0];
}

__device__ __forceinline__ float bjvp_point(float below, float cur, float above, float jm, float jp, float km, float kp,
                                            float cc, float h2inv) {
    float s = 6.0f * cur;
    s = s - below;
    s = s - above;
    s = s - jm;
    s = s - jp;
    s = s - km;
    s = s - kp;
    return h2inv * s - cc * cur;
}

// out = F'(x) v in FP32 arithmetic from an FP32 v (the V-cycle's output) and c32, at the
// instances with act[t] set: the single-instance FP32 product's arithmetic (two planes a step).
// eta (may be null): an instance whose forcing term is below tight takes the product to FP32 accuracy
// (jvp32xf_point: the stencil sum in double-FP32), as the single-instance path's tight linear solves do.
__global__ void __launch_bounds__(kBX* kBY) k_bjvp32f(const float* __restrict__ c32, const float* __restrict__ v,
                                                      float* __restrict__ out, const int* __restrict__ act, BClass C,
                                                      const double* __restrict__ eta, double tight) {
    pdl_wait();
    pdl_trigger();
    const int gq = blockIdx.z / C.zch, bz = blockIdx.z - gq * C.zch;
    if (!act[C.t0 + gq]) return;
    const bool precise = eta != nullptr && eta[C.t0 + gq] < tight;  // uniform over the block
    auto point = [precise](float below, float cur, float above, float jm, float jp, float km, float kp, float cc,
                           float h2inv) {
        return precise ? jvp32xf_point(below, cur, above, jm, jp, km, kp, cc, h2inv)
                       : bjvp_point(below, cur, above, jm, jp, km, kp, cc, h2inv);
    };
    const int n = C.n;
    const int k = blockIdx.x * kBX + threadIdx.x;
    const int j = blockIdx.y * kBY + threadIdx.y;
    if (k >= n || j >= n) return;
    const long long base = C.off0 + (long long)gq * C.N;
    c32 += base;
    v += base;
    out += base;
    const float h2inv = C.h2inv32;
    const int i0 = bz * C.ichunk;
    const int i1 = min(i0 + C.ichunk, n);
    const size_t plane = (size_t)n * n;
    const size_t col = (size_t)j * n + k;
    const bool jlo = j > 0, jhi = j + 1 < n, klo = k > 0, khi = k + 1 < n;
    float below = i0 > 0 ? v[(size_t)(i0 - 1) * plane + col] : 0.0f;
    float cur = i0 < i1 ? v[(size_t)i0 * plane + col] : 0.0f;
    int i = i0;
    for (; i + 1 < i1; i += 2) {
        const size_t p = (size_t)i * plane + col, q = p + plane;
        const float a1 = v[q];
        const float a2 = (i + 2 < n) ? v[q + plane] : 0.0f;
        const float jm0 = jlo ? v[p - n] : 0.0f, jp0 = jhi ? v[p + n] : 0.0f;
        const float km0 = klo ? v[p - 1] : 0.0f, kp0 = khi ? v[p + 1] : 0.0f;
        const float jm1 = jlo ? v[q - n] : 0.0f, jp1 = jhi ? v[q + n] : 0.0f;
        const float km1 = klo ? v[q - 1] : 0.0f, kp1 = khi ? v[q + 1] : 0.0f;
        const float c0 = c32[p], c1 = c32[q];
        out[p] = point(below, cur, a1, jm0, jp0, km0, kp0, c0, h2inv);
        out[q] = point(cur, a1, a2, jm1, jp1, km1, kp1, c1, h2inv);
        below = a1;
        cur = a2;
    }
    if (i < i1) {
        const size_t p = (size_t)i * plane + col;
        const float above = (i + 1 < n) ? v[p + plane] : 0.0f;
        const float jm = jlo ? v[p - n] : 0.0f, jp = jhi ? v[p + n] : 0.0f;
        const float km = klo ? v[p - 1] : 0.0f, kp = khi ? v[p + 1] : 0.0f;
        out[p] = point(below, cur, above, jm, jp, km, kp, c32[p], h2inv);
    }
}

// ------------------------------------------------------------------------------ element-wise passes
// Block table: block b covers elements [beg[b], end[b]) of the packed vectors, all of instance inst[b].
struct BlkTab {
    const int* inst;
    const long long* beg;
    const long long* end;
};

constexpr int kEwThreads = 256;
constexpr int kCgsBlock = 8;  // basis vectors per fused Gram-Schmidt / update pass

// Block reduction of R sums to partials[b * R + r] (thread 0).
template <int R>
__device__ __forceinline__ void block_partials(double (&s)[R], double* __restrict__ partials) {
    __shared__ double sm[R][32];
    block_sum<R>(s, sm);
    if (threadIdx.x == 0)
#pragma unroll
        for (int r = 0; r < R; ++r) partials[(size_t)blockIdx.x * R + r] = s[r];
}

// Per-instance FGMRES data, arrays of length I * stride.
struct BKry {
    double* hcol;   // Hessenberg column of the current step: the dots (0..j), then ||u_{j+1}||^2 (j+1)
    double* sig;    // 1/||u_r|| of the basis vectors (m + 1 per instance)
    double* sig2;   // 1/||u_r||^2
    double* coef;   // solution-update coefficients (m per instance), scaled to |c| <= 1
    double* scale;  // their scale (one per instance)
    int* kdone;     // basis vectors of the finished cycle (one per instance)
    int m1;         // m + 1 (the stride of sig, sig2 and hcol)
    int m;          // m (the stride of coef)
};

// h[r] = <w, u_{b0 + r}>, r < CNT, in double-FP32 (u_s at U + s T), partials per block.
template <int CNT>
__global__ void __launch_bounds__(kEwThreads) k_bdots(const float* __restrict__ w, const float* __restrict__ U,
                                                      long long T, int b0, BlkTab B, const int* __restrict__ act,
                                                      double* __restrict__ partials) {
    pdl_wait();
    pdl_trigger();
    const int t = B.inst[blockIdx.x];
    if (!act[t]) return;
    DF acc[CNT];
#pragma unroll
    for (int r = 0; r < CNT; ++r) acc[r] = DF{0.0f, 0.0f};
    const float* u = U + (long long)b0 * T;
    // UF elements a thread an iteration, all loads first (more DRAM bytes in flight), same order
    constexpr int UF = CNT <= 2 ? 8 : (CNT <= 3 ? 4 : 2);
    const long long e1 = B.end[blockIdx.x];
    long long i = B.beg[blockIdx.x] + threadIdx.x;
    for (; i + (UF - 1) * kEwThreads < e1; i += UF * kEwThreads) {
        float wv[UF], uv[UF][CNT];
#pragma unroll
        for (int q = 0; q < UF; ++q) {
            wv[q] = w[i + q * kEwThreads];
#pragma unroll
            for (int r = 0; r < CNT; ++r) uv[q][r] = u[(long long)r * T + i + q * kEwThreads];
        }
#pragma unroll
        for (int q = 0; q < UF; ++q)
#pragma unroll
            for (int r = 0; r < CNT; ++r) df_mac(acc[r], wv[q], uv[q][r]);
    }
    for (; i < e1; i += kEwThreads) {
        const float wi = w[i];
#pragma unroll
        for (int r = 0; r < CNT; ++r) df_mac(acc[r], wi, u[(long long)r * T + i]);
    }
    double s[CNT];
#pragma unroll
    for (int r = 0; r < CNT; ++r) s[r] = df_to_f64(acc[r]);
    block_partials<CNT>(s, partials);
}

// u_{j+1} = RN32(sigma_j (w - sum_{r<cnt} h_r sigma_r^2 u_r)) over the basis block b0 .. b0 + CNT - 1,
// the single-instance CGS1 update in double-FP32.  LAST = false: the partial sum goes to part (the
// earlier blocks of a basis longer than CNT); LAST: u_{j+1} is stored and ||u_{j+1}||^2 goes to the
// block's partial.  The first block starts from sigma_j w, later ones from part.
template <int CNT, bool LAST>
__global__ void __launch_bounds__(kEwThreads) k_bupdate(const float* __restrict__ w, float2* part,
                                                        float* __restrict__ U, long long T, int j, int b0, bool first,
                                                        BlkTab B, const int* __restrict__ act, BKry K,
                                                        double* __restrict__ partials) {
    pdl_wait();
    pdl_trigger();
    const int t = B.inst[blockIdx.x];
    if (!act[t]) return;
    const double* sig = K.sig + (long long)t * K.m1;
    const double* sig2 = K.sig2 + (long long)t * K.m1;
    const double* h = K.hcol + (long long)t * K.m1;
    const double a = sig[j];
    const DF cw = df_split(a);
    DF c[CNT];
#pragma unroll
    for (int r = 0; r < CNT; ++r) c[r] = df_split(-(a * h[b0 + r] * sig2[b0 + r]));
    const float* u = U + (long long)b0 * T;
    float* uout = U + (long long)(j + 1) * T;
    DF acc{0.0f, 0.0f};
    auto body = [&](long long i, float wi, float2 pv, const float (&ur)[CNT]) {
        DF s{0.0f, 0.0f};
        if (first) df_mac(s, cw, wi);
        else s = DF{pv.x, pv.y};
#pragma unroll
        for (int r = 0; r < CNT; ++r) df_mac(s, c[r], ur[r]);
        if (LAST) {
            const float v = __fadd_rn(s.hi, s.lo);
            uout[i] = v;
            df_mac(acc, v, v);
        } else {
            part[i] = make_float2(s.hi, s.lo);
        }
    };
    auto load = [&](long long i, float& wi, float2& pv, float (&ur)[CNT]) {
        if (first) wi = w[i];
        else pv = part[i];
#pragma unroll
        for (int r = 0; r < CNT; ++r) ur[r] = u[(long long)r * T + i];
    };
    // UF elements a thread an iteration, all loads first (more DRAM bytes in flight), same order; each
    // element of part is read before it is written, by one thread
    constexpr int UF = CNT <= 2 ? 8 : (CNT <= 3 ? 4 : 2);
    const long long e1 = B.end[blockIdx.x];
    long long i = B.beg[blockIdx.x] + threadIdx.x;
    for (; i + (UF - 1) * kEwThreads < e1; i += UF * kEwThreads) {
        float wv[UF] = {}, uv[UF][CNT];
        float2 pv[UF] = {};
#pragma unroll
        for (int q = 0; q < UF; ++q) load(i + q * kEwThreads, wv[q], pv[q], uv[q]);
#pragma unroll
        for (int q = 0; q < UF; ++q) body(i + q * kEwThreads, wv[q], pv[q], uv[q]);
    }
    for (; i < e1; i += kEwThreads) {
        float wi = 0.0f, ur[CNT];
        float2 pv = make_float2(0.0f, 0.0f);
        load(i, wi, pv, ur);
        body(i, wi, pv, ur);
    }
    if (LAST) {
        double sv[1] = {df_to_f64(acc)};
        block_partials<1>(sv, partials);
    }
}

// The solution update of the finished cycle over the basis block b0 .. b0 + CNT - 1:
// z (+)= scale sum_{r<kdone} coef_r Z_r (the first block assigns on a first cycle), and with the
// last block the full Newton step xn = x - z, where x is the instance's current iterate.
template <int CNT>
__global__ void __launch_bounds__(kEwThreads) k_bcombine(const float* __restrict__ Z, long long T, int b0, bool first,
                                                         bool last, double* __restrict__ z,
                                                         const double* __restrict__ xa, double* __restrict__ xb,
                                                         const int* __restrict__ cur, const int* __restrict__ act,
                                                         const int* __restrict__ assign, BlkTab B, BKry K) {
    pdl_wait();
    pdl_trigger();
    const int t = B.inst[blockIdx.x];
    if (!act[t]) return;
    const int kd = K.kdone[t];
    const double* cf = K.coef + (long long)t * K.m;
    const double sc = K.scale[t];
    DF c[CNT];
#pragma unroll
    for (int r = 0; r < CNT; ++r) c[r] = df_split(b0 + r < kd ? cf[b0 + r] : 0.0);
    const bool asg = first && assign[t] != 0;
    const double* x = cur[t] ? xb : xa;
    double* xn = cur[t] ? const_cast<double*>(xa) : xb;
    const float* Zb = Z + (long long)b0 * T;
    auto body = [&](long long i, const float (&zr)[CNT], double zi, double xi) {
        DF s{0.0f, 0.0f};
#pragma unroll
        for (int r = 0; r < CNT; ++r)
            if (b0 + r < kd) df_mac(s, c[r], zr[r]);
        const double v = asg ? __dmul_rn(sc, df_to_f64(s)) : __fma_rn(sc, df_to_f64(s), zi);
        z[i] = v;
        if (last) xn[i] = xi - v;
    };
    auto load = [&](long long i, float (&zr)[CNT], double& zi, double& xi) {
#pragma unroll
        for (int r = 0; r < CNT; ++r) zr[r] = b0 + r < kd ? Zb[(long long)r * T + i] : 0.0f;
        if (!asg) zi = z[i];
        if (last) xi = x[i];
    };
    // UF elements a thread an iteration, all loads first (more DRAM bytes in flight)
    constexpr int UF = CNT <= 2 ? 8 : (CNT <= 3 ? 4 : 2);
    const long long e1 = B.end[blockIdx.x];
    long long i = B.beg[blockIdx.x] + threadIdx.x;
    for (; i + (UF - 1) * kEwThreads < e1; i += UF * kEwThreads) {
        float zv[UF][CNT];
        double zs[UF] = {}, xs[UF] = {};
#pragma unroll
        for (int q = 0; q < UF; ++q) load(i + q * kEwThreads, zv[q], zs[q], xs[q]);
#pragma unroll
        for (int q = 0; q < UF; ++q) body(i + q * kEwThreads, zv[q], zs[q], xs[q]);
    }
    for (; i < e1; i += kEwThreads) {
        float zr[CNT];
        double zi = 0.0, xi = 0.0;
        load(i, zr, zi, xi);
        body(i, zr, zi, xi);
    }
}

// xn = x - alpha z (a line-search trial after a rejected one)
__global__ void __launch_bounds__(kEwThreads) k_bstep(const double* __restrict__ z, const double* __restrict__ xa,
                                                      double* __restrict__ xb, const int* __restrict__ cur,
                                                      const int* __restrict__ act, const double* __restrict__ alpha,
                                                      BlkTab B) {
    pdl_wait();
    pdl_trigger();
    const int t = B.inst[blockIdx.x];
    if (!act[t]) return;
    const double* x = cur[t] ? xb : xa;
    double* xn = cur[t] ? const_cast<double*>(xa) : xb;
    const double al = alpha[t];
    for (long long i = B.beg[blockIdx.x] + threadIdx.x; i < B.end[blockIdx.x]; i += kEwThreads) xn[i] = x[i] - al * z[i];
}

// restart of a cycle: v32 = RN32(z), the input of the FP32 product J z
__global__ void __launch_bounds__(kEwThreads) k_bto32(const double* __restrict__ z, float* __restrict__ v32,
                                                      const int* __restrict__ act, BlkTab B) {
    pdl_wait();
    pdl_trigger();
    const int t = B.inst[blockIdx.x];
    if (!act[t]) return;
    for (long long i = B.beg[blockIdx.x] + threadIdx.x; i < B.end[blockIdx.x]; i += kEwThreads) v32[i] = f64_to_f32(z[i]);
}

// restart: r = F - J z (FP64, the FP32 product widened) and ||r||^2 partials
__global__ void __launch_bounds__(kEwThreads) k_bsub(const double* __restrict__ F, const float* __restrict__ w,
                                                     double* __restrict__ r, const int* __restrict__ act, BlkTab B,
                                                     double* __restrict__ partials) {
    pdl_wait();
    pdl_trigger();
    const int t = B.inst[blockIdx.x];
    if (!act[t]) return;
    double s[1] = {0.0};
    for (long long i = B.beg[blockIdx.x] + threadIdx.x; i < B.end[blockIdx.x]; i += kEwThreads) {
        const double v = F[i] - f32_to_f64(w[i]);
        r[i] = v;
        s[0] = __fma_rn(v, v, s[0]);
    }
    block_partials<1>(s, partials);
}

// restart: u_0 = RN32(r / beta) (the new cycle's first FP32 basis vector, norm ~1)
__global__ void __launch_bounds__(kEwThreads) k_bscale32(const double* __restrict__ r, float* __restrict__ u0,
                                                         const double* __restrict__ inv_beta,
                                                         const int* __restrict__ act, BlkTab B) {
    pdl_wait();
    pdl_trigger();
    const int t = B.inst[blockIdx.x];
    if (!act[t]) return;
    const double s = inv_beta[t];
    for (long long i = B.beg[blockIdx.x] + threadIdx.x; i < B.end[blockIdx.x]; i += kEwThreads)
        u0[i] = f64_to_f32(__dmul_rn(r[i], s));
}

// Per-instance sums of block partials, in block order: out[t * ostride + ooff + r] = sum over the
// instance's partial slots [p0[t], p0[t] + pn[t]) of partials[slot * R + r], for r < R.  One warp per
// instance; lane r sums result r.
__global__ void k_bsegsum(const double* __restrict__ partials, int R, const int* __restrict__ p0,
                          const int* __restrict__ pn, const int* __restrict__ act, int I, double* __restrict__ out,
                          int ostride, int ooff) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (t >= I || !act[t] || lane >= R) return;
    double s = 0.0;
    const int b0 = p0[t], nb = pn[t];
    for (int b = 0; b < nb; ++b) s += partials[(size_t)(b0 + b) * R + lane];
    out[(long long)t * ostride + ooff + lane] = s;
}

}  // namespace
}  // namespace numa::gpu
