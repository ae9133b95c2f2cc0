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
//    Three passes over the basis, 4(j+1)+1 FP64 operations per point; for j+1 <= 16.
// On this GPU FP64 arithmetic, not bandwidth, bounds these kernels, so MGS is the cheaper of
// the two; CGS2 issues fewer launches and is the better-conditioned choice.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "numa_internal.hpp"

namespace numa::gpu {
namespace {

constexpr int kMaxCgs = 16;

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

// MODE 0: h[r] = <w, V_r>.
// MODE 1: w -= sum_r hin[r] V_r, then h[r] = <w, V_r>.
// MODE 2: w -= sum_r hin[r] V_r, then h[0] = ||w||.
template <int MODE>
__global__ void __launch_bounds__(kRedThreads) k_cgs(double* __restrict__ w, const double* __restrict__ V, size_t ldv,
                                                     int cnt, const double* __restrict__ hin, size_t N, RedArgs red,
                                                     double* __restrict__ hout) {
    __shared__ double sm[kMaxCgs][32];
    __shared__ double hs[kMaxCgs];
    if (MODE != 0 && threadIdx.x < kMaxCgs) hs[threadIdx.x] = threadIdx.x < (unsigned)cnt ? hin[threadIdx.x] : 0.0;
    __syncthreads();
    double s[kMaxCgs];
#pragma unroll
    for (int r = 0; r < kMaxCgs; ++r) s[r] = 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) {
        double wi = w[i];
        if (MODE != 0) {
            for (int r = 0; r < cnt; ++r) wi = __fma_rn(-hs[r], V[(size_t)r * ldv + i], wi);
            w[i] = wi;
        }
        if (MODE == 2) {
            s[0] = __fma_rn(wi, wi, s[0]);
        } else {
#pragma unroll
            for (int r = 0; r < kMaxCgs; ++r)
                if (r < cnt) s[r] = __fma_rn(wi, V[(size_t)r * ldv + i], s[r]);
        }
    }
    block_sum<kMaxCgs>(s, sm);
    const int nres = MODE == 2 ? 1 : cnt;
    grid_reduce_finish<kMaxCgs>(s, red, [hout, nres] __device__(const double(&t)[kMaxCgs]) {
        if (MODE == 2) hout[0] = __dsqrt_rn(t[0]);
        else for (int r = 0; r < nres; ++r) hout[r] = t[r];
    });
}

// dst = src / d (gmres.hpp:128, :149) as src * RN(1/d): one FP64 instruction instead of a
// division (within 1.5 ulp of it; the basis vectors already differ from the reference's in the
// last bits through the order of the inner-product sums).
__global__ void k_div(const double* __restrict__ src, double d, double rd, double* __restrict__ dst, size_t N) {
    (void)d;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) dst[i] = src[i] * rd;
}

// r = b - w (gmres.hpp:116)
__global__ void k_sub(const double* __restrict__ b, const double* __restrict__ w, double* __restrict__ r, size_t N) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) r[i] = b[i] - w[i];
}

// out = base + sum_i coef[i] * V_i, accumulated in i order per element as the reference's
// sequence of axpy calls does (gmres.hpp:198-199 with base = 0; :304-310 with base = b), each
// term fused into one FMA.
__global__ void k_combine(const double* __restrict__ base, const double* __restrict__ V, size_t ldv, int cnt,
                          const double* __restrict__ coef, double* __restrict__ out, size_t N) {
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
    k_mgs<false, false><<<g, kRedThreads, 0, ctx_.stream>>>(w, nullptr, nullptr, V, N, ctx_.red, StoreAt{hcol});
    ctx_.count_launch();
    for (size_t i = 1; i <= j; ++i) {
        k_mgs<true, false><<<g, kRedThreads, 0, ctx_.stream>>>(w, V + (i - 1) * N, hcol + (i - 1), V + i * N, N,
                                                              ctx_.red, StoreAt{hcol + i});
        ctx_.count_launch();
    }
    k_mgs<true, true><<<g, kRedThreads, 0, ctx_.stream>>>(w, V + j * N, hcol + j, nullptr, N, ctx_.red,
                                                         StoreSqrtAt{hcol + j + 1});
    ctx_.count_launch();
    ctx_.check_launch("arnoldi mgs");
}

void Gmres::arnoldi_cgs2(size_t j, double* w) {
    double* hcol = ctx_.scalar(kSlotGmresH);
    double* h2 = ctx_.scalar(kSlotGmresH2);
    const size_t N = N_;
    const unsigned g = ctx_.red_grid(N);
    const int cnt = (int)(j + 1);
    k_cgs<0><<<g, kRedThreads, 0, ctx_.stream>>>(w, V_.p, N, cnt, nullptr, N, ctx_.red, hcol);
    k_cgs<1><<<g, kRedThreads, 0, ctx_.stream>>>(w, V_.p, N, cnt, hcol, N, ctx_.red, h2);
    k_cgs<2><<<g, kRedThreads, 0, ctx_.stream>>>(w, V_.p, N, cnt, h2, N, ctx_.red, hcol + j + 1);
    ctx_.count_launch(3);
    ctx_.check_launch("arnoldi cgs2");
    // H = h + h' is formed on the host after the column is read (see solve).
}

GmresResult Gmres::solve(LinearOp& A, Precond* M, const double* b, double* x, const GmresOptions& o,
                         KrylovSpace* save, const double* r_init) {
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
            k_sub<<<eg, 256, 0, ctx_.stream>>>(b, w_.p, r_.p, N);
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
        k_div<<<eg, 256, 0, ctx_.stream>>>(rv, beta, 1.0 / beta, V_.p, N);
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
            if (cgs2 && j + 1 <= (size_t)kMaxCgs) {
                arnoldi_cgs2(j, w_.p);
                ctx_.fetch(sl, (int)(j + 2), col.data());
                ctx_.fetch(ctx_.scalar(kSlotGmresH2), (int)(j + 1), col2.data());
                for (size_t i = 0; i <= j; ++i) col[i] += col2[i];
            } else {
                arnoldi_mgs(j, w_.p);
                ctx_.fetch(sl, (int)(j + 2), col.data());
            }
            for (size_t i = 0; i <= j + 1; ++i) H[i][j] = col[i];
            double* vnext = V_.p + (j + 1) * N;
            if (H[j + 1][j] > 0.0) {
                k_div<<<eg, 256, 0, ctx_.stream>>>(w_.p, H[j + 1][j], 1.0 / H[j + 1][j], vnext, N);
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
            k_combine<<<eg, 256, k * sizeof(double), ctx_.stream>>>(nullptr, Z_.p, N, (int)k, ydev, comb_.p, N);
            ctx_.count_launch();
            dev_axpy(ctx_, 1.0, comb_.p, x, N);
        } else {
            k_combine<<<eg, 256, k * sizeof(double), ctx_.stream>>>(nullptr, V_.p, N, (int)k, ydev, comb_.p, N);
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
    k_combine<<<eg, 256, (k + 1) * sizeof(double), ctx_.stream>>>(b, sp.V.p, N, (int)(k + 1), cdev, rrec_.p, N);
    // comb = sum_{j<k} y_j V_j; x = M comb (gmres.hpp:312-317)
    k_combine<<<eg, 256, k * sizeof(double), ctx_.stream>>>(nullptr, sp.V.p, N, (int)k, cdev + k + 1, comb_.p, N);
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
