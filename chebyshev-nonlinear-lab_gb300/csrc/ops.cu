// ops.cu — the operator layer shared by every problem: workspaces, the finite-difference
// derivatives of operators/operator.hpp:101-134 over any NonlinearOp, and the Burgers2D
// operator (problems/burgers2d.hpp).
#include <cmath>
#include <limits>
#include <vector>

#include "numa_internal.hpp"

namespace numa::gpu {
namespace {

// ||v|| and the finite-difference step h = scale (1 + ||x||) / ||v|| on the device; a zero
// direction raises the flag that makes the quotient kernels write zeros (operator.hpp:105-106).
__global__ void __launch_bounds__(kRedThreads) k_fd_step(const double* __restrict__ v, size_t N, RedArgs red,
                                                         double scale, double* slots /* h, h^2, zero, xnorm, RN(1/h), RN(1/h^2) */) {
    __shared__ double sm[1][32];
    double s[1] = {0.0};
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) s[0] = __fma_rn(v[i], v[i], s[0]);
    block_sum<1>(s, sm);
    grid_reduce_finish<1>(s, red, [slots, scale] __device__(const double(&t)[1]) {
        const double nv = __dsqrt_rn(t[0]);
        if (nv == 0.0) {
            slots[0] = 0.0;
            slots[1] = 0.0;
            slots[2] = 1.0;
            slots[4] = 0.0;
            slots[5] = 0.0;
        } else {
            const double h = __ddiv_rn(scale * (1.0 + slots[3]), nv);
            slots[0] = h;
            slots[1] = h * h;
            slots[2] = 0.0;
            slots[4] = recip_for_div(h);          // kSlotFdInvH
            slots[5] = recip_for_div(slots[1]);   // kSlotFdInvHH
        }
    });
}

// xp = x + s h v with h from the device (s = +1 or -1): operator.hpp:109-110, :126-128.
__global__ void k_fd_shift(const double* __restrict__ x, const double* __restrict__ v, const double* __restrict__ slots,
                           double sign, double* __restrict__ xp, size_t N) {
    const double a = sign * slots[0];
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) xp[p] = x[p] + a * v[p];
}

// out = (f1 - f0) / h  (operator.hpp:113); the correctly rounded quotient from RN(1/h)
__global__ void k_fd_quot(const double* __restrict__ f1, const double* __restrict__ f0,
                          const double* __restrict__ slots, double* __restrict__ out, size_t N) {
    const double h = slots[0], rh = slots[4];
    const bool zero = slots[2] != 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride)
        out[p] = zero ? 0.0 : div_by_recip(f1[p] - f0[p], h, rh);
}

// out = (fp - 2 f0 + fm) / (h h)  (operator.hpp:132-133); the correctly rounded quotient from RN(1/h^2)
__global__ void k_fd2_quot(const double* __restrict__ fp, const double* __restrict__ f0, const double* __restrict__ fm,
                           const double* __restrict__ slots, double* __restrict__ out, size_t N) {
    const double hh = slots[1], rhh = slots[5];
    const bool zero = slots[2] != 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride)
        out[p] = zero ? 0.0 : div_by_recip(fp[p] - 2.0 * f0[p] + fm[p], hh, rhh);
}

unsigned ew_grid(const Context& ctx, size_t N) {
    size_t want = (N + 255) / 256;
    size_t cap = static_cast<size_t>(ctx.sm_count) * 16;
    if (want > cap) want = cap;
    return static_cast<unsigned>(want < 1 ? 1 : want);
}

// ------------------------------------------------------------------------------ Burgers2D kernels
// Component c of point (i, j) lives at c*n^2 + i*n + j; a neighbour outside the grid is 0.
struct BurgersGeom {
    int n;
    double inv2h, invh2, invdt, nu;
};

__device__ __forceinline__ double bat(const double* __restrict__ a, int n, size_t nn, int c, int i, int j) {
    return (i < 0 || j < 0 || i >= n || j >= n) ? 0.0 : a[c * nn + (size_t)i * n + j];
}

// F(w) = w/dt + (u u_x + v u_y, u v_x + v v_y) - nu Lap_h w - g  (burgers2d.hpp:169-210, :65-69),
// the reference's operation order term for term; optionally ||F||.
template <bool NORM>
__global__ void __launch_bounds__(256) k_burgers_eval(const double* __restrict__ w, const double* __restrict__ g,
                                                      double* __restrict__ out, BurgersGeom G, RedArgs red,
                                                      double* norm_out) {
    const int j = blockIdx.x * 32 + threadIdx.x;
    const int i = blockIdx.y * 8 + threadIdx.y;
    const int n = G.n;
    const size_t nn = (size_t)n * n;
    double acc[1] = {0.0};
    if (i < n && j < n) {
        const size_t p = (size_t)i * n + j;
        const double u = w[p], v = w[nn + p];
        const double ux = (bat(w, n, nn, 0, i, j + 1) - bat(w, n, nn, 0, i, j - 1)) * G.inv2h;
        const double uy = (bat(w, n, nn, 0, i + 1, j) - bat(w, n, nn, 0, i - 1, j)) * G.inv2h;
        const double vx = (bat(w, n, nn, 1, i, j + 1) - bat(w, n, nn, 1, i, j - 1)) * G.inv2h;
        const double vy = (bat(w, n, nn, 1, i + 1, j) - bat(w, n, nn, 1, i - 1, j)) * G.inv2h;
        const double lu = (bat(w, n, nn, 0, i, j + 1) + bat(w, n, nn, 0, i, j - 1) + bat(w, n, nn, 0, i + 1, j) +
                           bat(w, n, nn, 0, i - 1, j) - 4.0 * u) * G.invh2;
        const double lv = (bat(w, n, nn, 1, i, j + 1) + bat(w, n, nn, 1, i, j - 1) + bat(w, n, nn, 1, i + 1, j) +
                           bat(w, n, nn, 1, i - 1, j) - 4.0 * v) * G.invh2;
        double fu = G.invdt * u + u * ux + v * uy - G.nu * lu;
        double fv = G.invdt * v + u * vx + v * vy - G.nu * lv;
        if (g) {
            fu = fu - g[p];
            fv = fv - g[nn + p];
        }
        out[p] = fu;
        out[nn + p] = fv;
        if (NORM) acc[0] = __fma_rn(fv, fv, __fma_rn(fu, fu, acc[0]));
    }
    if (NORM) {
        __shared__ double sm[1][32];
        block_sum<1>(acc, sm);
        grid_reduce_finish<1>(acc, red, [norm_out] __device__(const double(&t)[1]) { *norm_out = __dsqrt_rn(t[0]); });
    }
}

// F'(w) d (burgers2d.hpp:71-123)
__global__ void __launch_bounds__(256) k_burgers_jvp(const double* __restrict__ w, const double* __restrict__ d,
                                                     double* __restrict__ out, BurgersGeom G) {
    const int j = blockIdx.x * 32 + threadIdx.x;
    const int i = blockIdx.y * 8 + threadIdx.y;
    const int n = G.n;
    if (i >= n || j >= n) return;
    const size_t nn = (size_t)n * n;
    const size_t p = (size_t)i * n + j;
    const double u = w[p], v = w[nn + p], du = d[p], dv = d[nn + p];
    const double ux = (bat(w, n, nn, 0, i, j + 1) - bat(w, n, nn, 0, i, j - 1)) * G.inv2h;
    const double uy = (bat(w, n, nn, 0, i + 1, j) - bat(w, n, nn, 0, i - 1, j)) * G.inv2h;
    const double vx = (bat(w, n, nn, 1, i, j + 1) - bat(w, n, nn, 1, i, j - 1)) * G.inv2h;
    const double vy = (bat(w, n, nn, 1, i + 1, j) - bat(w, n, nn, 1, i - 1, j)) * G.inv2h;
    const double dux = (bat(d, n, nn, 0, i, j + 1) - bat(d, n, nn, 0, i, j - 1)) * G.inv2h;
    const double duy = (bat(d, n, nn, 0, i + 1, j) - bat(d, n, nn, 0, i - 1, j)) * G.inv2h;
    const double dvx = (bat(d, n, nn, 1, i, j + 1) - bat(d, n, nn, 1, i, j - 1)) * G.inv2h;
    const double dvy = (bat(d, n, nn, 1, i + 1, j) - bat(d, n, nn, 1, i - 1, j)) * G.inv2h;
    const double ldu = (bat(d, n, nn, 0, i, j + 1) + bat(d, n, nn, 0, i, j - 1) + bat(d, n, nn, 0, i + 1, j) +
                        bat(d, n, nn, 0, i - 1, j) - 4.0 * du) * G.invh2;
    const double ldv = (bat(d, n, nn, 1, i, j + 1) + bat(d, n, nn, 1, i, j - 1) + bat(d, n, nn, 1, i + 1, j) +
                        bat(d, n, nn, 1, i - 1, j) - 4.0 * dv) * G.invh2;
    out[p] = G.invdt * du + du * ux + u * dux + dv * uy + v * duy - G.nu * ldu;
    out[nn + p] = G.invdt * dv + du * vx + u * dvx + dv * vy + v * dvy - G.nu * ldv;
}

// F''(w)[d, d] = 2 (du dux + dv duy, du dvx + dv dvy) (burgers2d.hpp:125-160)
__global__ void __launch_bounds__(256) k_burgers_d2(const double* __restrict__ d, double* __restrict__ out,
                                                    BurgersGeom G) {
    const int j = blockIdx.x * 32 + threadIdx.x;
    const int i = blockIdx.y * 8 + threadIdx.y;
    const int n = G.n;
    if (i >= n || j >= n) return;
    const size_t nn = (size_t)n * n;
    const size_t p = (size_t)i * n + j;
    const double du = d[p], dv = d[nn + p];
    const double dux = (bat(d, n, nn, 0, i, j + 1) - bat(d, n, nn, 0, i, j - 1)) * G.inv2h;
    const double duy = (bat(d, n, nn, 0, i + 1, j) - bat(d, n, nn, 0, i - 1, j)) * G.inv2h;
    const double dvx = (bat(d, n, nn, 1, i, j + 1) - bat(d, n, nn, 1, i, j - 1)) * G.inv2h;
    const double dvy = (bat(d, n, nn, 1, i + 1, j) - bat(d, n, nn, 1, i - 1, j)) * G.inv2h;
    out[p] = 2.0 * (du * dux + dv * duy);
    out[nn + p] = 2.0 * (du * dvx + dv * dvy);
}

}  // namespace

// ------------------------------------------------------------------------------ NonlinearOp
NonlinearOp::~NonlinearOp() = default;

SolverWorkspace& NonlinearOp::workspace() {
    if (!ws_) ws_ = std::make_unique<SolverWorkspace>(ctx_, size());
    return *ws_;
}

void NonlinearOp::jvp_fd(const double* x, const double* f0, const double* xnorm_dev, const double* v, double* out) {
    // h = sqrt(eps) (1 + ||x||) / ||v||; sqrt(eps) = 2^-26 exactly.
    const size_t N = size();
    double* slots = ctx_.scalar(kSlotFdH);
    dev_copy(ctx_, xnorm_dev, slots + 3, 1);
    const double scale = std::sqrt(std::numeric_limits<double>::epsilon());
    k_fd_step<<<ctx_.red_grid(N), kRedThreads, 0, ctx_.stream>>>(v, N, ctx_.red, scale, slots);
    ctx_.count_launch();
    fd1_.resize(N);
    fd2_.resize(N);
    k_fd_shift<<<ew_grid(ctx_, N), 256, 0, ctx_.stream>>>(x, v, slots, 1.0, fd1_.p, N);
    ctx_.count_launch();
    eval(fd1_.p, fd2_.p, nullptr, nullptr);
    k_fd_quot<<<ew_grid(ctx_, N), 256, 0, ctx_.stream>>>(fd2_.p, f0, slots, out, N);
    ctx_.count_launch();
    ctx_.check_launch("jvp_fd");
}

void NonlinearOp::d2_fd(const double* x, const double* f0, const double* xnorm_dev, const double* v, double* out) {
    // h = eps^(1/4) (1 + ||x||) / ||v||; eps^(1/4) = 2^-13 exactly.
    const size_t N = size();
    double* slots = ctx_.scalar(kSlotFdH);
    dev_copy(ctx_, xnorm_dev, slots + 3, 1);
    const double scale = std::pow(std::numeric_limits<double>::epsilon(), 0.25);
    k_fd_step<<<ctx_.red_grid(N), kRedThreads, 0, ctx_.stream>>>(v, N, ctx_.red, scale, slots);
    ctx_.count_launch();
    fd1_.resize(N);
    fd2_.resize(N);
    fd3_.resize(N);
    k_fd_shift<<<ew_grid(ctx_, N), 256, 0, ctx_.stream>>>(x, v, slots, 1.0, fd1_.p, N);
    ctx_.count_launch();
    eval(fd1_.p, fd2_.p, nullptr, nullptr);
    k_fd_shift<<<ew_grid(ctx_, N), 256, 0, ctx_.stream>>>(x, v, slots, -1.0, fd1_.p, N);
    ctx_.count_launch();
    eval(fd1_.p, fd3_.p, nullptr, nullptr);
    k_fd2_quot<<<ew_grid(ctx_, N), 256, 0, ctx_.stream>>>(fd2_.p, f0, fd3_.p, slots, out, N);
    ctx_.count_launch();
    ctx_.check_launch("d2_fd");
}

// ------------------------------------------------------------------------------ Burgers2D
// The manufactured root and the source g = F(w*) without source are formed on the host in
// double precision exactly as the reference does (burgers2d.hpp:25-52) and uploaded.
Burgers2D::Burgers2D(Context& ctx, size_t n, double nu, double dt, double amplitude)
    : NonlinearOp(ctx), n_(n), nu_(nu), dt_(dt), amp_(amplitude) {
    if (n == 0 || !(nu > 0.0) || !(dt > 0.0) || !std::isfinite(nu) || !std::isfinite(dt) || !std::isfinite(amplitude))
        throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "Burgers2D requires valid n, nu and dt");
    if (n > 46340) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "Burgers2D grid too large");
    const double h = 1.0 / (static_cast<double>(n) + 1.0);
    inv2h_ = 1.0 / (2.0 * h);
    invh2_ = 1.0 / (h * h);
    invdt_ = 1.0 / dt;
    const double pi = std::acos(-1.0);
    const size_t nn = n * n;
    std::vector<double> ex(2 * nn);
    for (size_t i = 0; i < n; ++i)
        for (size_t j = 0; j < n; ++j) {
            const double y = (static_cast<double>(i) + 1.0) * h;
            const double x = (static_cast<double>(j) + 1.0) * h;
            ex[i * n + j] = amplitude * std::sin(pi * x) * std::sin(pi * y);
            ex[nn + i * n + j] = amplitude * std::sin(2.0 * pi * x) * std::sin(pi * y);
        }
    exact_.resize(2 * nn);
    source_.resize(2 * nn);
    NUMA_CUDA(cudaMemcpyAsync(exact_.p, ex.data(), 2 * nn * sizeof(double), cudaMemcpyHostToDevice, ctx_.stream));
    // g = F_without_source(w*), on the device with the same arithmetic as every evaluation
    const BurgersGeom G{(int)n, inv2h_, invh2_, invdt_, nu_};
    const dim3 grid((unsigned)((n + 31) / 32), (unsigned)((n + 7) / 8));
    k_burgers_eval<false><<<grid, dim3(32, 8), 0, ctx_.stream>>>(exact_.p, nullptr, source_.p, G, ctx_.red, nullptr);
    ctx_.count_launch();
    ctx_.sync();
    ctx_.check_launch("Burgers2D setup");
}

void Burgers2D::eval(const double* x, double* out, double*, double* norm_out) {
    const BurgersGeom G{(int)n_, inv2h_, invh2_, invdt_, nu_};
    const dim3 grid((unsigned)((n_ + 31) / 32), (unsigned)((n_ + 7) / 8));
    // the fused norm needs one partial per block; larger grids take the norm separately
    const bool fused = norm_out && (size_t)grid.x * grid.y <= (size_t)kMaxRedBlocks;
    if (fused)
        k_burgers_eval<true><<<grid, dim3(32, 8), 0, ctx_.stream>>>(x, source_.p, out, G, ctx_.red, norm_out);
    else
        k_burgers_eval<false><<<grid, dim3(32, 8), 0, ctx_.stream>>>(x, source_.p, out, G, ctx_.red, nullptr);
    ctx_.count_launch();
    ctx_.check_launch("Burgers2D eval");
    if (norm_out && !fused) dev_norm2(ctx_, out, size(), norm_out);
}

void Burgers2D::jvp_at(const double* x, const double* v, double* out) {
    const BurgersGeom G{(int)n_, inv2h_, invh2_, invdt_, nu_};
    const dim3 grid((unsigned)((n_ + 31) / 32), (unsigned)((n_ + 7) / 8));
    k_burgers_jvp<<<grid, dim3(32, 8), 0, ctx_.stream>>>(x, v, out, G);
    ctx_.count_launch();
    ctx_.check_launch("Burgers2D jvp");
}

void Burgers2D::d2(const double*, const double*, const double* v, double* out) {
    const BurgersGeom G{(int)n_, inv2h_, invh2_, invdt_, nu_};
    const dim3 grid((unsigned)((n_ + 31) / 32), (unsigned)((n_ + 7) / 8));
    k_burgers_d2<<<grid, dim3(32, 8), 0, ctx_.stream>>>(v, out, G);
    ctx_.count_launch();
    ctx_.check_launch("Burgers2D d2");
}

}  // namespace numa::gpu
