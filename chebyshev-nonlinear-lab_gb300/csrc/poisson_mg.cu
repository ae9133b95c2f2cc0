// poisson_mg.cu — geometric-multigrid V-cycle for -Laplacian_h (linalg/poisson_mg.hpp) on the GPU.
//
// Same hierarchy as the reference: levels while n is odd, (n-1)/2 and h^-2/4 per level, down to
// n = 1 (poisson_mg.hpp:44-63); red-black Gauss-Seidel with colour (i+j+k)&1, order 0 = colour
// 0 then 1 for pre-smoothing and order 1 for post-smoothing (:99-126, :278-293); 27-point full
// weighting (:152-188); trilinear additive prolongation (:191-260); coarsest level exact at
// n = 1, else 30 alternating sweeps (:266-275).
//
// GB300 choices (FP64 is the scarce resource, ~1.2 TFLOP/s; FP32 runs at HBM speed):
//  * b h^2 is formed once per level and cycle (the reference recomputes b*inv in every sweep:
//    the stored product is the same rounded value);
//  * x / 6 uses the 3-operation correctly rounded division (div6);
//  * the first pass of a level, whose x is zero, reads no neighbours (they are +0.0), and no
//    level's x is zero-filled: every value the reference would read as zero is overwritten
//    before it is read;
//  * prolongation is added only at colour-0 points when post-smoothing follows: the first
//    post-smoothing pass overwrites every colour-1 point without reading it;
//  * the finest level of the FP64 cycle smooths directly in the output vector z and reads r in
//    place, so no copies in or out.
// The FP64 cycle reproduces the reference V-cycle bit for bit.  The FP32 cycle (precision
// extension) runs the same steps in single precision.
#include <cstring>
#include <limits>

#include "numa_internal.hpp"

namespace numa::gpu {

struct PoissonMG::Level {
    int n = 0;
    double h2inv = 0.0;
    double inv = 0.0;  // 1.0 / h2inv, as the reference forms it (poisson_mg.hpp:101)
    DeviceArray<double> x64, b64, bs64;
    DeviceArray<float> x32, b32, bs32;
};

namespace {

constexpr int BX = 32, BY = 8;

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
    if (OUT_Z) z[p] = (double)v;
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
    bsc[q] = (T)((double)acc * inv_c);
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

// b32 = (float) r, bs32 = (float)(r * inv) at the finest FP32 level.
__global__ void k_scale_in32(const double* __restrict__ r, float* __restrict__ b, float* __restrict__ bs, double inv,
                             size_t N) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) {
        const double v = r[p];
        b[p] = (float)v;
        bs[p] = (float)(v * inv);
    }
}

__global__ void k_to64(const float* __restrict__ x, double* __restrict__ z, size_t N) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) z[p] = (double)x[p];
}

// Coarsest level with one point: x = b / (6 h^-2) (poisson_mg.hpp:267-269).
template <class T>
__global__ void k_single(const T* __restrict__ b, T* __restrict__ x, double* __restrict__ z, double six_h2inv) {
    const T v = (T)((double)b[0] / six_h2inv);
    x[0] = v;
    if (z) z[0] = (double)v;
}

template <class T> T* xp(PoissonMG::Level& L);
template <> double* xp<double>(PoissonMG::Level& L) { return L.x64.p; }
template <> float* xp<float>(PoissonMG::Level& L) { return L.x32.p; }
template <class T> T* bp(PoissonMG::Level& L);
template <> double* bp<double>(PoissonMG::Level& L) { return L.b64.p; }
template <> float* bp<float>(PoissonMG::Level& L) { return L.b32.p; }
template <class T> T* bsp(PoissonMG::Level& L);
template <> double* bsp<double>(PoissonMG::Level& L) { return L.bs64.p; }
template <> float* bsp<float>(PoissonMG::Level& L) { return L.bs32.p; }

unsigned ew_grid(const Context& ctx, size_t N) {
    size_t want = (N + 255) / 256;
    size_t cap = static_cast<size_t>(ctx.sm_count) * 16;
    if (want > cap) want = cap;
    return static_cast<unsigned>(want < 1 ? 1 : want);
}

}  // namespace

PoissonMG::PoissonMG(Context& ctx, size_t n, int pre, int post, int precision, int max_levels)
    : ctx_(ctx), N0_(0), pre_(pre), post_(post), precision_(precision) {
    if (n == 0) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "PoissonMG requires a positive grid size");
    if (pre < 0 || post < 0) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "PoissonMG requires non-negative sweep counts");
    const size_t maxs = std::numeric_limits<size_t>::max();
    if (n > maxs / n || n * n > maxs / n) throw Status(NUMA_GPU_ERR_OVERFLOW, "PoissonMG cannot represent n^3");
    if (n > 65535) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "PoissonMG grid too large for one device");
    if (precision != NUMA_GPU_FP64 && precision != NUMA_GPU_FP32)
        throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "unknown precision");
    N0_ = n * n * n;
    size_t m = n;
    double h2 = (static_cast<double>(n) + 1.0) * (static_cast<double>(n) + 1.0);
    for (;;) {
        auto L = std::make_unique<Level>();
        L->n = static_cast<int>(m);
        L->h2inv = h2;
        L->inv = 1.0 / h2;
        const size_t Nl = m * m * m;
        const bool finest = levels_.empty();
        if (precision == NUMA_GPU_FP64) {
            L->bs64.resize(Nl);
            if (!finest) {
                L->x64.resize(Nl);
                L->b64.resize(Nl);
            }
        } else {
            L->x32.resize(Nl);
            L->b32.resize(Nl);
            L->bs32.resize(Nl);
        }
        levels_.push_back(std::move(L));
        if (m % 2 == 0 || m <= 1) break;
        if (max_levels > 0 && (int)levels_.size() >= max_levels) break;
        m = (m - 1) / 2;
        h2 /= 4.0;
    }
    if (levels_.size() > 1) {
        if (precision == NUMA_GPU_FP64) scratch_r_.resize(N0_);
        else scratch_r_.resize((N0_ + 1) / 2);  // N0 floats
    }
}

PoissonMG::~PoissonMG() = default;

template <class T>
void PoissonMG::cycle(size_t l) {
    Level& L = *levels_[l];
    const int n = L.n;
    const bool finest = (l == 0);
    T* x = finest ? static_cast<T*>(x0_) : xp<T>(L);
    const T* b = finest ? static_cast<const T*>(b0_) : bp<T>(L);
    const T* bs = finest ? static_cast<const T*>(bs0_) : bsp<T>(L);
    double* z = finest ? z0_ : nullptr;
    const size_t Nl = (size_t)n * n * n;
    cudaStream_t s = ctx_.stream;
    const dim3 blk(BX, BY);
    const dim3 cgrid(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, n);

    auto pass = [&](int colour, bool first, bool outz) {
        if (first && outz) k_rbgs<T, true, true><<<cgrid, blk, 0, s>>>(x, bs, z, n, colour);
        else if (first) k_rbgs<T, true, false><<<cgrid, blk, 0, s>>>(x, bs, nullptr, n, colour);
        else if (outz) k_rbgs<T, false, true><<<cgrid, blk, 0, s>>>(x, bs, z, n, colour);
        else k_rbgs<T, false, false><<<cgrid, blk, 0, s>>>(x, bs, nullptr, n, colour);
        ctx_.count_launch();
    };
    // order 0: colour 0 then 1; order 1: colour 1 then 0 (poisson_mg.hpp:103-106)
    auto sweep = [&](int order, bool first, bool outz) {
        const int c0 = order == 0 ? 0 : 1;
        pass(c0, first, outz);
        pass(1 - c0, false, outz);
    };

    if (l + 1 == levels_.size()) {
        if (n == 1) {
            k_single<T><<<1, 1, 0, s>>>(b, x, z, 6.0 * L.h2inv);
            ctx_.count_launch();
        } else {
            for (int sw = 0; sw < 30; ++sw) sweep(sw % 2, sw == 0, z != nullptr && sw == 29);
        }
        ctx_.check_launch("mg coarsest");
        return;
    }

    for (int sw = 0; sw < pre_; ++sw) sweep(0, sw == 0, false);
    if (pre_ == 0) NUMA_CUDA(cudaMemsetAsync(x, 0, Nl * sizeof(T), s));

    T* r = reinterpret_cast<T*>(scratch_r_.p);
    {
        const int ichunk = n >= 64 ? 8 : 1;
        const dim3 g((n + BX - 1) / BX, (n + BY - 1) / BY, (n + ichunk - 1) / ichunk);
        k_residual<T><<<g, blk, 0, s>>>(x, b, r, n, ichunk, (T)L.h2inv);
        ctx_.count_launch();
    }
    Level& C = *levels_[l + 1];
    const int nc = C.n;
    {
        const dim3 g((nc + BX - 1) / BX, (nc + BY - 1) / BY, nc);
        k_restrict<T><<<g, blk, 0, s>>>(r, bp<T>(C), bsp<T>(C), n, nc, C.inv);
        ctx_.count_launch();
    }
    ctx_.check_launch("mg restrict");
    cycle<T>(l + 1);
    if (post_ > 0) {
        const dim3 g(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, n);
        k_prolong<T, true><<<g, blk, 0, s>>>(xp<T>(C), x, nc, n);
    } else {
        const dim3 g((n + BX - 1) / BX, (n + BY - 1) / BY, n);
        k_prolong<T, false><<<g, blk, 0, s>>>(xp<T>(C), x, nc, n);
    }
    ctx_.count_launch();
    for (int sw = 0; sw < post_; ++sw) sweep(1, false, z != nullptr && sw == post_ - 1);
    if (z != nullptr && post_ == 0) {
        k_to64<<<ew_grid(ctx_, Nl), 256, 0, s>>>(reinterpret_cast<const float*>(x), z, Nl);
        ctx_.count_launch();
    }
    ctx_.check_launch("mg cycle");
}

void PoissonMG::apply(const double* r, double* z) {
    Level& L0 = *levels_[0];
    const size_t N = N0_;
    if (precision_ == NUMA_GPU_FP64) {
        const double* b = r;
        if (r == z) {
            alias_b_.resize(N);
            dev_copy(ctx_, r, alias_b_.p, N);
            b = alias_b_.p;
        }
        k_scale_in64<<<ew_grid(ctx_, N), 256, 0, ctx_.stream>>>(b, L0.bs64.p, L0.inv, N);
        ctx_.count_launch();
        x0_ = z;
        b0_ = b;
        bs0_ = L0.bs64.p;
        z0_ = nullptr;
        cycle<double>(0);
    } else {
        k_scale_in32<<<ew_grid(ctx_, N), 256, 0, ctx_.stream>>>(r, L0.b32.p, L0.bs32.p, L0.inv, N);
        ctx_.count_launch();
        x0_ = L0.x32.p;
        b0_ = L0.b32.p;
        bs0_ = L0.bs32.p;
        z0_ = z;
        cycle<float>(0);
    }
    ctx_.check_launch("mg apply");
}

double PoissonMG::time_finest_pass(int reps) {
    Level& L0 = *levels_[0];
    const int n = L0.n;
    const size_t N = N0_;
    const dim3 blk(BX, BY);
    const dim3 cgrid(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, n);
    cudaEvent_t a, b;
    NUMA_CUDA(cudaEventCreate(&a));
    NUMA_CUDA(cudaEventCreate(&b));
    float ms = 0.f;
    if (precision_ == NUMA_GPU_FP64) {
        DeviceArray<double> x(N);
        NUMA_CUDA(cudaMemsetAsync(x.p, 0, N * sizeof(double), ctx_.stream));
        NUMA_CUDA(cudaMemsetAsync(L0.bs64.p, 0, N * sizeof(double), ctx_.stream));
        k_rbgs<double, false, false><<<cgrid, blk, 0, ctx_.stream>>>(x.p, L0.bs64.p, nullptr, n, 0);
        NUMA_CUDA(cudaEventRecord(a, ctx_.stream));
        for (int r = 0; r < reps; ++r)
            k_rbgs<double, false, false><<<cgrid, blk, 0, ctx_.stream>>>(x.p, L0.bs64.p, nullptr, n, r & 1);
        NUMA_CUDA(cudaEventRecord(b, ctx_.stream));
        NUMA_CUDA(cudaEventSynchronize(b));
    } else {
        NUMA_CUDA(cudaMemsetAsync(L0.x32.p, 0, N * sizeof(float), ctx_.stream));
        NUMA_CUDA(cudaMemsetAsync(L0.bs32.p, 0, N * sizeof(float), ctx_.stream));
        k_rbgs<float, false, false><<<cgrid, blk, 0, ctx_.stream>>>(L0.x32.p, L0.bs32.p, nullptr, n, 0);
        NUMA_CUDA(cudaEventRecord(a, ctx_.stream));
        for (int r = 0; r < reps; ++r)
            k_rbgs<float, false, false><<<cgrid, blk, 0, ctx_.stream>>>(L0.x32.p, L0.bs32.p, nullptr, n, r & 1);
        NUMA_CUDA(cudaEventRecord(b, ctx_.stream));
        NUMA_CUDA(cudaEventSynchronize(b));
    }
    ctx_.count_launch(reps + 1);
    NUMA_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    ctx_.check_launch("time_finest_pass");
    return reps > 0 ? ms / reps : 0.0;
}

}  // namespace numa::gpu
