// drivers.cu — preconditioner providers and the nonlinear drivers newton_krylov,
// chebyshev_inexact (methods/krylov_newton.hpp) and tf_chebyshev_2018
// (methods/tf_chebyshev_2018.hpp) with every vector on the device.
//
// The control flow, counters, forcing terms, line searches and acceptance tests are the
// reference's, statement for statement; only the vector work runs as kernels, and each scalar
// the host decides on (a norm) is read back once.  The drivers run on any NonlinearOp
// (Bratu3D, Burgers2D).  An operator's per-iterate cache (for Bratu3D the coefficient
// c = lambda e^x) is produced by the residual evaluation of x itself and reused by every
// Jacobian product, F''(x)[z,z] and the Jacobi diagonal at that iterate.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "numa_internal.hpp"

namespace numa::gpu {
namespace {

// ------------------------------------------------------------------------------ providers
class IdentityProvider : public Provider {
public:
    IdentityProvider(Context& ctx, size_t N) : ctx_(ctx), N_(N) {}
    void make(const double*, const double*) override {}
    void apply(const double* r, double* z) override { dev_copy(ctx_, r, z, N_); }
    int kind() const override { return NUMA_GPU_PRECOND_NONE; }

private:
    Context& ctx_;
    size_t N_;
};

class MGProvider : public Provider {
public:
    MGProvider(Context& ctx, size_t n, int pre, int post, int precision, int max_levels)
        : mg_(ctx, n, pre, post, precision, max_levels) {}
    void make(const double*, const double*) override {}  // PoissonMGProvider::make ignores x
    void apply(const double* r, double* z) override { mg_.apply(r, z); }
    // the FP32 cycle can hand its result over unwidened
    bool has_apply32() const override { return mg_.supports_out32(); }
    void apply32(const double* r, float* z32) override { mg_.apply32(r, z32); }
    bool has_apply32f() const override { return mg_.supports_out32(); }
    void apply32f(const float* r32, float* z32) override { mg_.apply32f(r32, z32); }
    int kind() const override { return NUMA_GPU_PRECOND_POISSON_MG; }
    PoissonMG& mg() { return mg_; }

private:
    PoissonMG mg_;
};

// The FP32 V-cycle with Jacobian-aware coarse levels, bound at each iterate: make() restricts the
// iterate's coefficient c = lambda e^x (the operator's cache) down to the one-CTA tail.
class JacobianMGProvider : public Provider {
public:
    JacobianMGProvider(Context& ctx, size_t n, int pre, int post) : mg_(ctx, n, pre, post, NUMA_GPU_FP32, 0) {
        if (!mg_.supports_coarse_jacobian() || !mg_.supports_out32())
            throw Status(NUMA_GPU_ERR_NOT_SUPPORTED,
                         "Jacobian-aware multigrid: the grid needs an odd hierarchy down to a tail of n <= 15");
    }
    void make(const double*, const double* c) override {
        if (!c) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "Jacobian-aware multigrid: the operator keeps no coefficient");
        mg_.set_coarse_coefficient(c);
    }
    void make_c32(const double*, const double* c, const float* c32) override { mg_.set_coarse_coefficient(c, c32); }
    void apply(const double* r, double* z) override { mg_.apply(r, z); }
    bool has_apply32() const override { return true; }
    void apply32(const double* r, float* z32) override { mg_.apply32(r, z32); }
    bool has_apply32f() const override { return true; }
    void apply32f(const float* r32, float* z32) override { mg_.apply32f(r32, z32); }
    int kind() const override { return NUMA_GPU_PRECOND_JACOBIAN_MG; }

private:
    PoissonMG mg_;
};

__global__ void k_jacobi_apply(const double* __restrict__ r, const double* __restrict__ d, double* __restrict__ z,
                               size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) z[i] = r[i] / d[i];
}

class JacobiProvider : public Provider {
public:
    explicit JacobiProvider(Bratu3D& op) : op_(op), d_(op.size()), c_(0) {}
    void make(const double* x, const double* c) override {
        if (!c) {
            c_.resize(op_.size());
            op_.coef(x, c_.p);
            c = c_.p;
        }
        op_.jacobi_diag_c(c, d_.p);
    }
    void apply(const double* r, double* z) override {
        Context& ctx = op_.ctx();
        const size_t N = op_.size();
        size_t g = (N + 255) / 256, cap = (size_t)ctx.sm_count * 16;
        launch_pdl(k_jacobi_apply, (unsigned)std::max<size_t>(1, std::min(g, cap)), 256, 0, ctx.stream, r, d_.p, z, N);
        ctx.count_launch();
        ctx.check_launch("jacobi apply");
    }
    int kind() const override { return NUMA_GPU_PRECOND_JACOBI; }

private:
    Bratu3D& op_;
    DeviceArray<double> d_, c_;
};

// ------------------------------------------------------------------------------ timers
// Per-primitive CUDA-event timers (operators/timing.hpp:16-24).  Off unless the context asks.
enum TimerKind { kT_F = 0, kT_JVP, kT_D2, kT_PREC, kT_SETUP, kT_N };

class Timers {
public:
    explicit Timers(Context& ctx) : ctx_(ctx) {}
    ~Timers() {
        for (auto e : pool_) cudaEventDestroy(e);
    }
    struct Scope {
        Timers* t;
        int kind;
        cudaEvent_t a = nullptr, b = nullptr;
        Scope(Timers* tt, int k) : t(tt), kind(k) {
            if (t->ctx_.timing) {
                a = t->take();
                NUMA_CUDA(cudaEventRecord(a, t->ctx_.stream));
            }
        }
        ~Scope() {
            if (a) {
                b = t->take();
                cudaEventRecord(b, t->ctx_.stream);
                t->pairs_.push_back({kind, a, b});
            }
        }
    };
    void collect(numa_krylov_result& out) {
        double acc[kT_N] = {0, 0, 0, 0, 0};
        if (!pairs_.empty()) {
            NUMA_CUDA(cudaStreamSynchronize(ctx_.stream));
            for (auto& p : pairs_) {
                float ms = 0.f;
                NUMA_CUDA(cudaEventElapsedTime(&ms, p.a, p.b));
                acc[p.kind] += ms * 1e-3;
            }
        }
        out.t_F = acc[kT_F];
        out.t_JVP = acc[kT_JVP];
        out.t_D2 = acc[kT_D2];
        out.t_prec = acc[kT_PREC];
        out.t_setup_dynamic = acc[kT_SETUP];
    }

private:
    struct Pair {
        int kind;
        cudaEvent_t a, b;
    };
    cudaEvent_t take() {
        if (used_ == pool_.size()) {
            cudaEvent_t e;
            NUMA_CUDA(cudaEventCreate(&e));
            pool_.push_back(e);
        }
        return pool_[used_++];
    }
    Context& ctx_;
    std::vector<cudaEvent_t> pool_;
    size_t used_ = 0;
    std::vector<Pair> pairs_;
};

// ------------------------------------------------------------------------------ Jacobian operator
// apply(v, out) = F'(x) v at the bound iterate x (krylov_newton.hpp:86): the operator's analytic
// product bound at x (FP64, or FP32 arithmetic where the operator offers it), or finite
// differences.
class JacobianOp : public LinearOp {
public:
    JacobianOp(NonlinearOp& f, Timers& t, int mode) : f_(f), t_(t), mode_(mode) {}
    void bind(const double* x, const double* fx, const double* xnorm) {
        x_ = x;
        fx_ = fx;
        xnorm_ = xnorm;
    }
    void apply(const double* v, double* out) override {
        Timers::Scope s(&t_, kT_JVP);
        if (mode_ == NUMA_GPU_DERIV_FD) f_.jvp_fd(x_, fx_, xnorm_, v, out);
        else f_.jvp_bound(v, out);
    }
    bool has_apply32() const override { return mode_ != NUMA_GPU_DERIV_FD && f_.has_jvp32(); }
    void apply32(const float* v32, double* out) override {
        Timers::Scope s(&t_, kT_JVP);
        f_.jvp_bound32(v32, out);
    }
    bool has_apply32f() const override { return mode_ != NUMA_GPU_DERIV_FD && f_.has_jvp32f(); }
    void apply32f(const float* v32, float* out32) override {
        Timers::Scope s(&t_, kT_JVP);
        f_.jvp_bound32f(v32, out32);
    }
    bool has_apply32x() const override { return mode_ != NUMA_GPU_DERIV_FD && f_.has_jvp32x(); }
    void apply32x(const float* v32, double* out) override {
        Timers::Scope s(&t_, kT_JVP);
        f_.jvp_bound32x(v32, out);
    }
    void apply32xf(const float* v32, float* out32) override {
        Timers::Scope s(&t_, kT_JVP);
        f_.jvp_bound32xf(v32, out32);
    }

private:
    NonlinearOp& f_;
    Timers& t_;
    int mode_;
    const double *x_ = nullptr, *fx_ = nullptr, *xnorm_ = nullptr;
};

class TimedPrecond : public Precond {
public:
    TimedPrecond(Provider* p, Timers& t) : p_(p), t_(t) {}
    void apply(const double* r, double* z) override {
        Timers::Scope s(&t_, kT_PREC);
        p_->apply(r, z);
    }
    void progress(size_t iters, double rel_res) override { p_->progress(iters, rel_res); }
    bool has_apply32() const override { return p_->has_apply32(); }
    void apply32(const double* r, float* z32) override {
        Timers::Scope s(&t_, kT_PREC);
        p_->apply32(r, z32);
    }
    bool has_apply32f() const override { return p_->has_apply32f(); }
    void apply32f(const float* r32, float* z32) override {
        Timers::Scope s(&t_, kT_PREC);
        p_->apply32f(r32, z32);
    }

private:
    Provider* p_;
    Timers& t_;
};

// (j1 - j0) / h  (tf_chebyshev_2018.hpp:46-48)
__global__ void k_quot(const double* __restrict__ a, const double* __restrict__ b, double h, double* __restrict__ out,
                       size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) out[i] = (a[i] - b[i]) / h;
}

unsigned ew_grid(const Context& ctx, size_t N) {
    size_t want = (N + 255) / 256;
    size_t cap = static_cast<size_t>(ctx.sm_count) * 16;
    if (want > cap) want = cap;
    return static_cast<unsigned>(want < 1 ? 1 : want);
}

// Shared state of a nonlinear solve: the iterate, its residual and operator cache, and the
// trial point, swapped by pointer on acceptance (x = xn; Fx = Fn).
struct SolveState {
    NonlinearOp& f;
    Context& ctx;
    const KrylovParams& p;
    size_t N;
    double* user_x;
    SolverWorkspace& W;
    DeviceArray<double>&xb, &Fa, &Fb, &ca, &cb, &z, &u, &w, &scratch, &xnorm;
    Gmres& gmres;
    double *x, *xn, *Fx, *Fn, *cx, *cn;
    Timers timers;

    SolveState(NonlinearOp& f_, const KrylovParams& p_, double* x0)
        : f(f_), ctx(f_.ctx()), p(p_), N(f_.size()), user_x(x0), W(f_.workspace()), xb(W.xb), Fa(W.Fa), Fb(W.Fb),
          ca(W.ca), cb(W.cb), z(W.z), u(W.u), w(W.w), scratch(W.scratch), xnorm(W.xnorm), gmres(W.gmres),
          timers(f_.ctx()) {
        xb.resize(N);
        Fa.resize(N);
        Fb.resize(N);
        f.prepare_cache(p.jvp_mode == NUMA_GPU_DERIV_ANALYTIC ? p.jvp_precision : NUMA_GPU_FP64);
        const size_t nc = f.cache_size();
        if (nc) {
            ca.resize(nc);
            cb.resize(nc);
        }
        z.resize(N);
        xnorm.resize(1);
        x = user_x;
        xn = xb.p;
        Fx = Fa.p;
        Fn = Fb.p;
        cx = nc ? ca.p : nullptr;
        cn = nc ? cb.p : nullptr;
    }
    // F(xn) with its coefficient and norm; returns ||F(xn)||.
    // RN32(F(x)) where the operator keeps it beside its FP32 Jacobian data (the FP32 hand-off)
    const float* f32() const {
        return p.jvp_precision == NUMA_GPU_FP32 && p.jvp_mode == NUMA_GPU_DERIV_ANALYTIC ? f.f32_of_cache(cx) : nullptr;
    }
    double eval_trial() {
        {
            Timers::Scope s(&timers, kT_F);
            f.eval(xn, Fn, cn, ctx.scalar(kSlotNormF));
        }
        return ctx.fetch1(ctx.scalar(kSlotNormF));
    }
    void accept() {
        std::swap(x, xn);
        std::swap(Fx, Fn);
        std::swap(cx, cn);
    }
    // Binds the Jacobian operator and the provider at the current iterate (make(x) timed as
    // dynamic setup, timing.hpp:98-103).
    void bind(JacobianOp& J, Provider* pc) {
        if (p.jvp_mode == NUMA_GPU_DERIV_ANALYTIC) f.bind(x, cx, p.jvp_precision);
        if (p.jvp_mode == NUMA_GPU_DERIV_FD || p.d2_mode == NUMA_GPU_DERIV_FD) dev_norm2(ctx, x, N, xnorm.p);
        J.bind(x, Fx, xnorm.p);
        if (pc) {
            Timers::Scope s(&timers, kT_SETUP);
            const float* c32 = f.coef32_of_cache(cx);
            if (c32) pc->make_c32(x, cx, c32);
            else pc->make(x, cx);
        }
    }
    // Copies the final iterate into the caller's vector if the swaps left it elsewhere.
    void finish() {
        if (x != user_x) dev_copy(ctx, x, user_x, N);
        ctx.sync();
    }
};

GmresOptions gmres_opts(const KrylovParams& p, double rtol, double bnorm = -1.0, const float* b32 = nullptr) {
    GmresOptions o;
    o.bnorm = bnorm;
    o.b32 = b32;
    o.rtol = rtol;
    o.restart = p.restart;
    o.max_iters = p.max_iters;
    o.zero_guess = true;
    o.orth = p.orth;
    o.flexible = p.flexible;
    o.precise_tight = p.jvp_tight;
    return o;
}

void add_lin(numa_krylov_result& out, const GmresResult& g) {
    out.n_JVP += g.matvecs;
    out.n_lin_iters += g.iters;
    out.n_prec += g.precs;
    if (!g.converged) ++out.n_lin_failures;
}

}  // namespace

// ------------------------------------------------------------------------------ factories
std::unique_ptr<Provider> make_identity_provider(Context& ctx, size_t N) {
    return std::make_unique<IdentityProvider>(ctx, N);
}
std::unique_ptr<Provider> make_mg_provider(Context& ctx, size_t n, int pre, int post, int precision, int max_levels) {
    return std::make_unique<MGProvider>(ctx, n, pre, post, precision, max_levels);
}
std::unique_ptr<Provider> make_jacobi_provider(Bratu3D& op) { return std::make_unique<JacobiProvider>(op); }
std::unique_ptr<Provider> make_jacobian_mg_provider(Context& ctx, size_t n, int pre, int post) {
    return std::make_unique<JacobianMGProvider>(ctx, n, pre, post);
}

KrylovParams params_from_c(const numa_krylov_params* c) {
    KrylovParams p;
    if (!c) return p;
    p.rtol_nl = c->rtol_nl;
    p.max_nl = c->max_nl;
    p.eta_init = c->eta_init;
    p.eta_max = c->eta_max;
    p.gamma = c->gamma;
    p.alpha = c->alpha;
    p.eta2_factor = c->eta2_factor;
    p.eta2_max = c->eta2_max;
    p.restart = c->gmres_restart;
    p.max_iters = c->gmres_max_iters;
    p.armijo = c->armijo;
    p.min_lambda = c->min_lambda;
    p.recycle = c->recycle != 0;
    p.jvp_mode = c->jvp_mode;
    p.d2_mode = c->d2_mode;
    p.orth = c->orth;
    p.flexible = c->flexible != 0;
    p.jvp_precision = c->jvp_precision;
    p.jvp_tight = c->jvp_tight != 0;
    p.coarse_jacobian = c->coarse_jacobian != 0;
    return p;
}

// Eisenstat-Walker choice 2 with Kelley's safeguard and the oversolve floor
// (krylov_newton.hpp:54-65).
double forcing(const KrylovParams& p, size_t k, double rnorm, double rprev, double eta_prev, double res0) {
    if (k == 0) return p.eta_init;
    double eta = p.gamma * std::pow(rnorm / rprev, p.alpha);
    const double safe = p.gamma * std::pow(eta_prev, p.alpha);
    if (safe > 0.1) eta = std::max(eta, safe);
    eta = std::min(eta, p.eta_max);
    eta = std::max(eta, 0.5 * p.rtol_nl * res0 / rnorm);
    return std::min(eta, p.eta_max);
}

// ------------------------------------------------------------------------------ newton_krylov
// krylov_newton.hpp:69-114
// *out = sqrt(sum of the K pieces' sums of squares), summed in piece order
__global__ void k_sum_sqrt(const double* __restrict__ parts, int K, double* __restrict__ out) {
    pdl_wait();
    pdl_trigger();
    double s = 0.0;
    for (int c = 0; c < K; ++c) s += parts[c];
    *out = __dsqrt_rn(s);
}

void newton_krylov(NonlinearOp& f, double* x0, const KrylovParams& p, Provider* pc, numa_krylov_result& out,
                   HostUpload* up) {
    const auto t0 = std::chrono::steady_clock::now();
    std::memset(&out, 0, sizeof(out));
    SolveState S(f, p, x0);
    JacobianOp J(f, S.timers, p.jvp_mode);
    TimedPrecond M(pc, S.timers);
    Precond* Mp = pc ? &M : nullptr;
    const size_t N = S.N;
    {
        Timers::Scope s(&S.timers, kT_F);
        const int K = up && up->host ? f.eval_pieces() : 0;
        if (up && up->host && K == 0) {
            NUMA_CUDA(cudaMemcpyAsync(S.x, up->host, N * sizeof(double), cudaMemcpyHostToDevice, S.ctx.stream));
        }
        if (K > 0) {
            // the pieces of x0 go up on the copy stream while the evaluation runs on those already there
            NUMA_CUDA(cudaEventRecord(up->start, S.ctx.stream));
            NUMA_CUDA(cudaStreamWaitEvent(up->copy, up->start, 0));
            for (int c = 0; c < K; ++c) {
                const size_t b0 = f.eval_piece_begin(c), b1 = c + 1 < K ? f.eval_piece_begin(c + 1) : N;
                NUMA_CUDA(cudaMemcpyAsync(S.x + b0, up->host + b0, (b1 - b0) * sizeof(double), cudaMemcpyHostToDevice,
                                          up->copy));
                NUMA_CUDA(cudaEventRecord(up->done[c], up->copy));
            }
            double* sums = S.ctx.scalar(kSlotPieceSums);
            for (int c = 0; c < K; ++c) {
                const size_t need = f.eval_piece_need(c);
                int last = c;  // the last piece whose upload the evaluation of piece c reads
                while (last + 1 < K && f.eval_piece_begin(last + 1) < need) ++last;
                NUMA_CUDA(cudaStreamWaitEvent(S.ctx.stream, up->done[last], 0));
                f.eval_piece(S.x, S.Fx, S.cx, c, sums + c);
            }
            launch_pdl(k_sum_sqrt, 1, 1, 0, S.ctx.stream, (const double*)sums, K, S.ctx.scalar(kSlotNormF));
            S.ctx.count_launch();
            S.ctx.check_launch("newton_krylov staged evaluation");
        } else {
            f.eval(S.x, S.Fx, S.cx, S.ctx.scalar(kSlotNormF));
        }
    }
    ++out.n_F;
    double rnorm = S.ctx.fetch1(S.ctx.scalar(kSlotNormF));
    out.res0 = rnorm;
    double rprev = rnorm, eta_prev = p.eta_init;
    const double* fetched = nullptr;  // the device iterate last downloaded to up->host_out
    for (size_t k = 0; k < p.max_nl; ++k) {
        if (rnorm <= p.rtol_nl * out.res0) {
            out.converged = 1;
            break;
        }
        fetched = nullptr;  // this iteration's step overwrites the other buffer, the next one this one
        const double eta = forcing(p, k, rnorm, rprev, eta_prev, out.res0);
        S.bind(J, pc);
        GmresOptions go = gmres_opts(p, eta, rnorm, S.f32());
        go.x_base = S.x;  // the solution update may form the full step xn = x - z in the same pass
        go.x_step = S.xn;
        const GmresResult g = S.gmres.solve(J, Mp, S.Fx, S.z.p, go);
        add_lin(out, g);
        if (g.breakdown) break;
        double lam = 1.0;
        bool ok = false;
        while (lam >= p.min_lambda) {
            if (!(lam == 1.0 && g.stepped)) dev_newton_step(S.ctx, S.x, S.z.p, lam, S.xn, N);
            // the linear model predicts the full step converges: download it while its residual is evaluated
            const bool fetch = up && up->host_out && lam == 1.0 && g.rel_res * rnorm <= p.rtol_nl * out.res0;
            if (fetch) {
                NUMA_CUDA(cudaEventRecord(up->fetch_start, S.ctx.stream));
                NUMA_CUDA(cudaStreamWaitEvent(up->copy, up->fetch_start, 0));
                NUMA_CUDA(cudaMemcpyAsync(up->host_out, S.xn, N * sizeof(double), cudaMemcpyDeviceToHost, up->copy));
                NUMA_CUDA(cudaEventRecord(up->fetch_done, up->copy));
                fetched = S.xn;
            }
            const double fn = S.eval_trial();
            ++out.n_F;
            if (fetch) NUMA_CUDA(cudaStreamWaitEvent(S.ctx.stream, up->fetch_done, 0));  // before xn is written again
            if (fn <= (1.0 - p.armijo * lam) * rnorm) {
                ok = true;
                rprev = rnorm;
                rnorm = fn;
                break;
            }
            fetched = nullptr;
            lam *= 0.5;
        }
        if (!ok) break;
        S.accept();
        eta_prev = eta;
        ++out.iters;
    }
    if (rnorm <= p.rtol_nl * out.res0) out.converged = 1;
    out.res = rnorm;
    if (up) up->fetched = fetched != nullptr && fetched == S.x;  // the returned iterate is the one downloaded
    S.finish();
    S.timers.collect(out);
    out.t_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// ------------------------------------------------------------------------------ chebyshev_inexact
// krylov_newton.hpp:116-189
void chebyshev_inexact(NonlinearOp& f, double* x0, const KrylovParams& p, Provider* pc, numa_krylov_result& out) {
    const auto t0 = std::chrono::steady_clock::now();
    std::memset(&out, 0, sizeof(out));
    SolveState S(f, p, x0);
    JacobianOp J(f, S.timers, p.jvp_mode);
    TimedPrecond M(pc, S.timers);
    Precond* Mp = pc ? &M : nullptr;
    const size_t N = S.N;
    S.u.resize(N);
    S.w.resize(N);
    KrylovSpace& space = S.W.space;
    {
        Timers::Scope s(&S.timers, kT_F);
        f.eval(S.x, S.Fx, S.cx, S.ctx.scalar(kSlotNormF));
    }
    ++out.n_F;
    double rnorm = S.ctx.fetch1(S.ctx.scalar(kSlotNormF));
    out.res0 = rnorm;
    double rprev = rnorm, eta_prev = p.eta_init;
    for (size_t k = 0; k < p.max_nl; ++k) {
        if (rnorm <= p.rtol_nl * out.res0) {
            out.converged = 1;
            break;
        }
        const double eta1 = forcing(p, k, rnorm, rprev, eta_prev, out.res0);
        const double eta2 = std::min(p.eta2_max, p.eta2_factor * eta1);
        S.bind(J, pc);
        space.clear();
        const GmresResult g1 =
            S.gmres.solve(J, Mp, S.Fx, S.z.p, gmres_opts(p, eta1, rnorm, S.f32()), p.recycle ? &space : nullptr);
        add_lin(out, g1);
        if (g1.breakdown) break;
        {
            Timers::Scope s(&S.timers, kT_D2);
            if (p.d2_mode == NUMA_GPU_DERIV_FD) f.d2_fd(S.x, S.Fx, S.xnorm.p, S.z.p, S.w.p);
            else f.d2(S.x, S.cx, S.z.p, S.w.p);
        }
        ++out.n_D2;
        const GmresResult g2 = p.recycle ? S.gmres.solve_recycled(J, Mp, S.w.p, S.u.p, gmres_opts(p, eta2), space)
                                         : S.gmres.solve(J, Mp, S.w.p, S.u.p, gmres_opts(p, eta2));
        add_lin(out, g2);
        bool ok = false;
        double fn_acc = 0.0;
        if (!g2.breakdown) {
            dev_cheb_step(S.ctx, S.x, S.z.p, S.u.p, S.xn, N);
            const double fn = S.eval_trial();
            ++out.n_F;
            if (fn < rnorm) {
                ok = true;
                fn_acc = fn;
            }
        }
        if (!ok) {
            double lam = 1.0;
            while (lam >= p.min_lambda) {
                dev_newton_step(S.ctx, S.x, S.z.p, lam, S.xn, N);
                const double fn = S.eval_trial();
                ++out.n_F;
                if (fn <= (1.0 - p.armijo * lam) * rnorm) {
                    ok = true;
                    fn_acc = fn;
                    break;
                }
                lam *= 0.5;
            }
        }
        if (!ok) break;
        S.accept();
        rprev = rnorm;
        rnorm = fn_acc;
        eta_prev = eta1;
        ++out.iters;
    }
    if (rnorm <= p.rtol_nl * out.res0) out.converged = 1;
    out.res = rnorm;
    S.finish();
    S.timers.collect(out);
    out.t_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// ------------------------------------------------------------------------------ tf_chebyshev_2018
// methods/tf_chebyshev_2018.hpp:52-132
void tf_chebyshev_2018(NonlinearOp& f, double* x0, const KrylovParams& p, Provider* pc, numa_krylov_result& out) {
    const auto t0 = std::chrono::steady_clock::now();
    std::memset(&out, 0, sizeof(out));
    SolveState S(f, p, x0);
    JacobianOp J(f, S.timers, p.jvp_mode);
    TimedPrecond M(pc, S.timers);
    Precond* Mp = pc ? &M : nullptr;
    Context& ctx = S.ctx;
    const size_t N = S.N;
    S.u.resize(N);      // d2 (second correction)
    S.w.resize(N);      // curvature / rhs2
    S.scratch.resize(2 * N);
    double* j0 = S.scratch.p;
    double* j1 = S.scratch.p + N;
    {
        Timers::Scope s(&S.timers, kT_F);
        f.eval(S.x, S.Fx, S.cx, ctx.scalar(kSlotNormF));
    }
    ++out.n_F;
    double rnorm = ctx.fetch1(ctx.scalar(kSlotNormF));
    out.res0 = rnorm;
    const double eps = std::numeric_limits<double>::epsilon();
    double* sl = ctx.scalar(kSlotTmp0);
    for (size_t k = 0; k < p.max_nl; ++k) {
        if (rnorm <= p.rtol_nl * out.res0) {
            out.converged = 1;
            break;
        }
        const double eta1 = std::clamp(std::min(1e-8, rnorm * rnorm), 2.0 * eps, 1e-8);
        const double eta2 = std::clamp(std::min(1e-8, rnorm), 2.0 * eps, 1e-8);
        S.bind(J, pc);
        const GmresResult g1 = S.gmres.solve(J, Mp, S.Fx, S.z.p, gmres_opts(p, eta1, rnorm, S.f32()));
        add_lin(out, g1);
        if (!g1.converged) break;
        if (g1.breakdown) break;
        // d1 = -z (in place: z is not needed afterwards)
        double* d1 = S.z.p;
        dev_scale_inplace(ctx, d1, -1.0, N);
        // h = clamp(sqrt(eps) ||x|| / ||d1||, 2 eps, 0.5) (tf_chebyshev_2018.hpp:23-29)
        dev_norm2(ctx, d1, N, sl);
        dev_norm2(ctx, S.x, N, sl + 1);
        double nrm[2];
        ctx.fetch(sl, 2, nrm);
        double h = 2.0 * eps;
        if (nrm[0] > 0.0) h = std::clamp(std::sqrt(eps) * nrm[1] / nrm[0], 2.0 * eps, 0.5);
        // xh = x + h d1 into xn; curvature = (J(xh) d1 - J(x) d1) / h
        dev_copy(ctx, S.x, S.xn, N);
        dev_axpy(ctx, h, d1, S.xn, N);
        {
            Timers::Scope s(&S.timers, kT_JVP);
            if (p.jvp_mode == NUMA_GPU_DERIV_FD) {
                f.jvp_fd(S.x, S.Fx, S.xnorm.p, d1, j0);
                f.eval(S.xn, S.Fn, nullptr, nullptr);  // F(xh), recomputed inside jvp_fd by the reference
                dev_norm2(ctx, S.xn, N, sl + 2);
                f.jvp_fd(S.xn, S.Fn, sl + 2, d1, j1);
            } else {
                // FP64 products whatever the Krylov product's precision: the curvature is a
                // difference quotient at h ~ sqrt(eps)
                f.jvp_cached(S.x, S.cx, d1, j0);
                f.jvp_at(S.xn, d1, j1);
            }
        }
        out.n_JVP += 2;
        launch_pdl(k_quot, ew_grid(ctx, N), 256, 0, ctx.stream, j1, j0, h, S.w.p, N);
        ctx.count_launch();
        dev_scale_inplace(ctx, S.w.p, -0.5, N);
        const GmresResult g2 = S.gmres.solve(J, Mp, S.w.p, S.u.p, gmres_opts(p, eta2));
        add_lin(out, g2);
        if (!g2.converged) break;
        if (g2.breakdown) break;
        // x += d1; x += d2 (in place on the iterate), then F(x)
        dev_axpy(ctx, 1.0, d1, S.x, N);
        dev_axpy(ctx, 1.0, S.u.p, S.x, N);
        {
            Timers::Scope s(&S.timers, kT_F);
            f.eval(S.x, S.Fx, S.cx, ctx.scalar(kSlotNormF));
        }
        ++out.n_F;
        rnorm = ctx.fetch1(ctx.scalar(kSlotNormF));
        ++out.iters;
        if (!std::isfinite(rnorm)) break;
    }
    if (rnorm <= p.rtol_nl * out.res0) out.converged = 1;
    out.res = rnorm;
    S.finish();
    S.timers.collect(out);
    out.t_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace numa::gpu
