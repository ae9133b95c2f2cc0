// hmg2d.cu — the 2D geometric-multigrid V-cycle for alpha I - nu Lap_h
// (linalg/helmholtz_mg2d.hpp) and the Burgers2D preconditioner provider built on it
// (problems/burgers2d.hpp:220-246), FP64.
//
// Same hierarchy (levels while n is odd, s = nu h^-2 quartered per level), red-black
// Gauss-Seidel with colour (i+j)&1 and the reference's colour orders, 9-point full weighting,
// bilinear additive prolongation, coarsest level exact at n = 1 else 30 alternating sweeps.  The
// arithmetic follows the reference operation for operation (the neighbour sum starts from 0.0,
// the update divides by alpha + 4s), so the cycle equals the reference's bit for bit.  As in the
// 3D cycle, the first colour pass of a level reads no neighbours (its x is zero there), and the
// prolongation is added only at colour-0 points when post-smoothing follows.
#include <limits>

#include "numa_internal.hpp"

namespace numa::gpu {

struct HelmholtzMG2D::Level {
    int n = 0;
    double s = 0.0;  // nu / h^2 of this level
    DeviceArray<double> x, b;
};

namespace {

constexpr int BX = 32, BY = 8;

// x = (b + s * nb) / (alpha + 4 s), nb = 0 + x_{i-1} + x_{i+1} + x_{j-1} + x_{j+1}
// (helmholtz_mg2d.hpp:51-70).  FIRST: x is zero before the pass.
template <bool FIRST>
__global__ void k_hsmooth(double* __restrict__ x, const double* __restrict__ b, int n, double s, double den,
                          int colour) {
    const int jj = blockIdx.x * BX + threadIdx.x;
    const int i = blockIdx.y * BY + threadIdx.y;
    if (i >= n) return;
    const int j = 2 * jj + ((i + colour) & 1);
    if (j >= n) return;
    const size_t p = (size_t)i * n + j;
    double nb = 0.0;
    if (!FIRST) {
        if (i > 0) nb = nb + x[p - n];
        if (i + 1 < n) nb = nb + x[p + n];
        if (j > 0) nb = nb + x[p - 1];
        if (j + 1 < n) nb = nb + x[p + 1];
    }
    x[p] = (b[p] + s * nb) / den;
}

// r = b - (alpha x + s (4x - nb)) (helmholtz_mg2d.hpp:72-87)
__global__ void k_hresidual(const double* __restrict__ x, const double* __restrict__ b, double* __restrict__ r, int n,
                            double s, double alpha) {
    const int j = blockIdx.x * BX + threadIdx.x;
    const int i = blockIdx.y * BY + threadIdx.y;
    if (i >= n || j >= n) return;
    const size_t p = (size_t)i * n + j;
    double nb = 0.0;
    if (i > 0) nb = nb + x[p - n];
    if (i + 1 < n) nb = nb + x[p + n];
    if (j > 0) nb = nb + x[p - 1];
    if (j + 1 < n) nb = nb + x[p + 1];
    r[p] = b[p] - (alpha * x[p] + s * (4.0 * x[p] - nb));
}

// coarse b = sum_{a,b} (w_a w_b) r(2I+a, 2J+b), weights (1/4,1/2,1/4) (helmholtz_mg2d.hpp:89-108);
// each weight product is a power of two, so the FMA equals the reference's multiply-then-add.
__global__ void k_hrestrict(const double* __restrict__ rf, double* __restrict__ bc, int nf, int nc) {
    const int J = blockIdx.x * BX + threadIdx.x;
    const int I = blockIdx.y * BY + threadIdx.y;
    if (I >= nc || J >= nc) return;
    const double w[3] = {0.25, 0.5, 0.25};
    double acc = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int fi = 2 * I + a;
        if (fi >= nf) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int fj = 2 * J + c;
            if (fj >= nf) continue;
            acc = __fma_rn(w[a] * w[c], rf[(size_t)fi * nf + fj], acc);
        }
    }
    bc[(size_t)I * nc + J] = acc;
}

__device__ __forceinline__ int hinterp(int f, int nc, int (&idx)[2]) {
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

// fine x += bilinear interpolation of coarse x (helmholtz_mg2d.hpp:110-136); COLOUR0_ONLY:
// only points with (i+j) even.
template <bool COLOUR0_ONLY>
__global__ void k_hprolong(const double* __restrict__ xc, double* __restrict__ xf, int nc, int nf) {
    const int t = blockIdx.x * BX + threadIdx.x;
    const int i = blockIdx.y * BY + threadIdx.y;
    if (i >= nf) return;
    const int j = COLOUR0_ONLY ? 2 * t + (i & 1) : t;
    if (j >= nf) return;
    int ci[2], cj[2];
    const int ni = hinterp(i, nc, ci), nj = hinterp(j, nc, cj);
    const double wi = (ni == 1 && (i & 1)) ? 1.0 : 0.5;
    const double wj = (nj == 1 && (j & 1)) ? 1.0 : 0.5;
    double acc = 0.0;
    for (int a = 0; a < ni; ++a)
        for (int c = 0; c < nj; ++c) acc = __fma_rn(wi * wj, xc[(size_t)ci[a] * nc + cj[c]], acc);
    const size_t p = (size_t)i * nf + j;
    xf[p] = xf[p] + acc;
}

// coarsest n = 1: x = b / (alpha + 4 s)
__global__ void k_hsingle(const double* __restrict__ b, double* __restrict__ x, double den) { x[0] = b[0] / den; }

}  // namespace

HelmholtzMG2D::HelmholtzMG2D(Context& ctx, size_t n, double alpha, double nu, int pre, int post)
    : ctx_(ctx), N0_(n * n), alpha_(alpha), pre_(pre), post_(post) {
    if (n == 0) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "HelmholtzMG2D requires a positive grid size");
    if (pre < 0 || post < 0) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "negative sweep count");
    if (n > 46340) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "HelmholtzMG2D grid too large");
    size_t m = n;
    double s = nu * (static_cast<double>(n) + 1.0) * (static_cast<double>(n) + 1.0);
    for (;;) {
        auto L = std::make_unique<Level>();
        L->n = static_cast<int>(m);
        L->s = s;
        if (!levels_.empty()) {
            L->x.resize(m * m);
            L->b.resize(m * m);
        }
        levels_.push_back(std::move(L));
        if (m % 2 == 0 || m <= 1) break;
        m = (m - 1) / 2;
        s /= 4.0;
    }
    resid_.resize(N0_);
}

HelmholtzMG2D::~HelmholtzMG2D() = default;

void HelmholtzMG2D::cycle(size_t l) {
    Level& L = *levels_[l];
    const int n = L.n;
    double* x = l == 0 ? x0_ : L.x.p;
    const double* b = l == 0 ? b0_ : L.b.p;
    const double den = alpha_ + 4.0 * L.s;
    cudaStream_t st = ctx_.stream;
    const dim3 blk(BX, BY);
    const dim3 cg(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY);
    auto pass = [&](int colour, bool first) {
        if (first) k_hsmooth<true><<<cg, blk, 0, st>>>(x, b, n, L.s, den, colour);
        else k_hsmooth<false><<<cg, blk, 0, st>>>(x, b, n, L.s, den, colour);
        ctx_.count_launch();
    };
    auto sweep = [&](int order, bool first) {
        const int c0 = order == 0 ? 0 : 1;
        pass(c0, first);
        pass(1 - c0, false);
    };
    if (l + 1 == levels_.size()) {
        if (n == 1) {
            k_hsingle<<<1, 1, 0, st>>>(b, x, den);
            ctx_.count_launch();
        } else {
            for (int sw = 0; sw < 30; ++sw) sweep(sw % 2, sw == 0);
        }
        ctx_.check_launch("hmg2d coarsest");
        return;
    }
    for (int sw = 0; sw < pre_; ++sw) sweep(0, sw == 0);
    if (pre_ == 0) NUMA_CUDA(cudaMemsetAsync(x, 0, (size_t)n * n * sizeof(double), st));
    const dim3 fg((n + BX - 1) / BX, (n + BY - 1) / BY);
    k_hresidual<<<fg, blk, 0, st>>>(x, b, resid_.p, n, L.s, alpha_);
    Level& C = *levels_[l + 1];
    const int nc = C.n;
    k_hrestrict<<<dim3((nc + BX - 1) / BX, (nc + BY - 1) / BY), blk, 0, st>>>(resid_.p, C.b.p, n, nc);
    ctx_.count_launch(2);
    cycle(l + 1);
    if (post_ > 0) k_hprolong<true><<<cg, blk, 0, st>>>(C.x.p, x, nc, n);
    else k_hprolong<false><<<fg, blk, 0, st>>>(C.x.p, x, nc, n);
    ctx_.count_launch();
    for (int sw = 0; sw < post_; ++sw) sweep(1, false);
    ctx_.check_launch("hmg2d cycle");
}

void HelmholtzMG2D::apply(const double* r, double* z) {
    const double* b = r;
    if (r == z) {
        alias_.resize(N0_);
        dev_copy(ctx_, r, alias_.p, N0_);
        b = alias_.p;
    }
    x0_ = z;
    b0_ = b;
    cycle(0);
}

namespace {

// BurgersMGProvider: M^-1 applied to u and v separately (burgers2d.hpp:228-243), in place on
// the two halves of the vectors.
class BurgersMGProvider : public Provider {
public:
    BurgersMGProvider(Context& ctx, size_t n, double nu, double dt, int pre, int post)
        : mg_(ctx, n, 1.0 / dt, nu, pre, post), nn_(n * n) {}
    void make(const double*, const double*) override {}
    void apply(const double* r, double* z) override {
        mg_.apply(r, z);
        mg_.apply(r + nn_, z + nn_);
    }
    int kind() const override { return NUMA_GPU_PRECOND_POISSON_MG; }

private:
    HelmholtzMG2D mg_;
    size_t nn_;
};

}  // namespace

std::unique_ptr<Provider> make_burgers_mg_provider(Context& ctx, size_t n, double nu, double dt, int pre, int post) {
    return std::make_unique<BurgersMGProvider>(ctx, n, nu, dt, pre, post);
}

}  // namespace numa::gpu
