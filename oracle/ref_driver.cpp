// ref_driver.cpp — C entry points over the reference's own headers (namespace numa::op).
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.sh against the reference's
// include/ directory where it lies (nothing of it is copied here) into oracle/_ref/libnuma_ref.so.
// tests/golden/make_golden.py loads that library to produce the committed golden fixtures that
// pin the CPU restatement in oracle/numa_oracle.cpp.  The reference is not present where the GPU
// tests run, so only the fixtures travel.
//
// Every function forwards to the reference template it names; the only code of this file is
// argument marshalling and an operator adaptor that routes jvp/d2 to the reference's own
// finite-difference forms (operators/operator.hpp:101-134).

#include <numa/linalg/gmres.hpp>
#include <numa/linalg/poisson_mg.hpp>
#include <numa/methods/krylov_newton.hpp>
#include <numa/methods/tf_chebyshev_2018.hpp>
#include <numa/operators/operator.hpp>
#include <numa/problems/bratu3d.hpp>
#include <numa/problems/brusselator1d.hpp>
#include <numa/problems/burgers2d.hpp>
#include <numa/linalg/helmholtz_mg2d.hpp>

#include "../include/numa_gpu.h"

#include <cstring>
#include <stdexcept>

using namespace numa::op;

namespace {

// Bratu3D with jvp / d2 replaced by jvp_fd / d2_fd of the same problem.
struct FdBratu {
    const Bratu3D& f;
    int jvp_mode;
    int d2_mode;
    std::size_t size() const { return f.size(); }
    void eval(const DVec& x, DVec& out) const { f.eval(x, out); }
    void jvp(const DVec& x, const DVec& v, DVec& out) const {
        if (jvp_mode == 1) jvp_fd(f, x, v, out); else f.jvp(x, v, out);
    }
    void d2(const DVec& x, const DVec& v, DVec& out) const {
        if (d2_mode == 1) d2_fd(f, x, v, out); else f.d2(x, v, out);
    }
};

KrylovParams to_params(const numa_krylov_params* cp) {
    KrylovParams p;
    if (!cp) return p;
    p.rtol_nl = cp->rtol_nl;
    p.max_nl = cp->max_nl;
    p.eta_init = cp->eta_init;
    p.eta_max = cp->eta_max;
    p.gamma = cp->gamma;
    p.alpha = cp->alpha;
    p.eta2_factor = cp->eta2_factor;
    p.eta2_max = cp->eta2_max;
    p.gmres_restart = cp->gmres_restart;
    p.gmres_max_iters = cp->gmres_max_iters;
    p.armijo = cp->armijo;
    p.min_lambda = cp->min_lambda;
    p.recycle = cp->recycle != 0;
    return p;
}

void fill(const GmresResult& g, numa_gmres_result* o) {
    if (!o) return;
    o->iters = g.iters;
    o->matvecs = g.matvecs;
    o->precs = g.precs;
    o->rel_res = g.rel_res;
    o->converged = g.converged;
    o->breakdown = g.breakdown;
}

template <class Op, class Prov>
KrylovResult run(int method, const Op& op, const DVec& x0, KrylovParams p, const Prov& pc) {
    if (method == NUMA_GPU_METHOD_NK) return newton_krylov(op, x0, p, pc);
    if (method == NUMA_GPU_METHOD_TF2018) return tf_chebyshev_2018(op, x0, p, pc);
    if (method == NUMA_GPU_METHOD_CHEB_REC) p.recycle = true;
    return chebyshev_inexact(op, x0, p, pc);
}

}  // namespace

extern "C" {

void ref_bratu3d_eval(size_t n, double lambda, const double* u, double* out) {
    Bratu3D f(n, lambda);
    DVec U(u, u + f.size()), O;
    f.eval(U, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
}

void ref_bratu3d_jvp(size_t n, double lambda, const double* u, const double* v, double* out, int mode) {
    Bratu3D f(n, lambda);
    DVec U(u, u + f.size()), V(v, v + f.size()), O;
    if (mode == 1) jvp_fd(f, U, V, O); else f.jvp(U, V, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
}

void ref_bratu3d_d2(size_t n, double lambda, const double* u, const double* v, double* out, int mode) {
    Bratu3D f(n, lambda);
    DVec U(u, u + f.size()), V(v, v + f.size()), O;
    if (mode == 1) d2_fd(f, U, V, O); else f.d2(U, V, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
}

void ref_bratu3d_jacobi_diag(size_t n, double lambda, const double* u, double* d) {
    Bratu3D f(n, lambda);
    DVec U(u, u + f.size()), D;
    f.jacobi_diag(U, D);
    std::memcpy(d, D.data(), D.size() * sizeof(double));
}

int ref_mg_levels(size_t n, int pre, int post) {
    try {
        PoissonMG mg(n, pre, post);
        return static_cast<int>(mg.levels());
    } catch (const std::overflow_error&) {
        return -2;
    } catch (const std::invalid_argument&) {
        return -1;
    }
}

int ref_mg_apply(size_t n, int pre, int post, const double* r, double* z) {
    PoissonMG mg(n, pre, post);
    DVec R(r, r + n * n * n), Z;
    mg(R, Z);
    std::memcpy(z, Z.data(), Z.size() * sizeof(double));
    return 0;
}

int ref_gmres_bratu3d(size_t n, double lambda, const double* xpt, int jvp_mode, int precond_kind,
                      const double* b, double* x, double rtol, size_t restart, size_t max_iters,
                      int zero_guess, numa_gmres_result* out) {
    Bratu3D f(n, lambda);
    FdBratu op{f, jvp_mode, 0};
    const std::size_t N = f.size();
    DVec X(xpt, xpt + N), B(b, b + N), S(x, x + N);
    auto A = [&](const DVec& v, DVec& o) { op.jvp(X, v, o); };
    GmresResult g;
    if (precond_kind == NUMA_GPU_PRECOND_POISSON_MG) {
        PoissonMGProvider pc(n);
        g = gmres(A, pc.make(X), B, S, rtol, restart, max_iters, zero_guess != 0);
    } else if (precond_kind == NUMA_GPU_PRECOND_JACOBI) {
        BratuJacobi pc{f};
        g = gmres(A, pc.make(X), B, S, rtol, restart, max_iters, zero_guess != 0);
    } else {
        g = gmres(A, IdentityPrecond{}, B, S, rtol, restart, max_iters, zero_guess != 0);
    }
    std::memcpy(x, S.data(), N * sizeof(double));
    fill(g, out);
    return 0;
}

int ref_gmres_recycle_pair(size_t n, double lambda, const double* xpt, int precond_kind,
                           const double* b1, const double* b2, double rtol, size_t restart,
                           size_t max_iters, double* z1, double* u2, size_t* k_saved,
                           numa_gmres_result* r1, numa_gmres_result* r2) {
    Bratu3D f(n, lambda);
    const std::size_t N = f.size();
    DVec X(xpt, xpt + N), B1(b1, b1 + N), B2(b2, b2 + N), Z(N, 0.0), U;
    auto A = [&](const DVec& v, DVec& o) { f.jvp(X, v, o); };
    KrylovSpace sp;
    GmresResult g1, g2;
    if (precond_kind == NUMA_GPU_PRECOND_POISSON_MG) {
        PoissonMG mg(n);
        g1 = gmres(A, mg, B1, Z, rtol, restart, max_iters, true, &sp);
        g2 = gmres_recycled(A, mg, B2, U, rtol, restart, max_iters, sp);
    } else {
        BratuJacobi pc{f};
        auto M = pc.make(X);
        g1 = gmres(A, M, B1, Z, rtol, restart, max_iters, true, &sp);
        g2 = gmres_recycled(A, M, B2, U, rtol, restart, max_iters, sp);
    }
    std::memcpy(z1, Z.data(), N * sizeof(double));
    std::memcpy(u2, U.data(), N * sizeof(double));
    if (k_saved) *k_saved = sp.k;
    fill(g1, r1);
    fill(g2, r2);
    return 0;
}

int ref_gmres_poisson_mg(size_t n, const double* b, double* x, double rtol, size_t restart,
                         size_t max_iters, numa_gmres_result* out) {
    // -Laplacian_h as Bratu3D's jvp at lambda = 0 (the same 7-point operator as the reference
    // test's apply_poisson, tests/test_operators.cpp:162-185).
    Bratu3D lap(n, 0.0);
    const std::size_t N = n * n * n;
    DVec zero(N, 0.0), B(b, b + N), S(N, 0.0);
    PoissonMG mg(n);
    auto A = [&](const DVec& v, DVec& o) { lap.jvp(zero, v, o); };
    GmresResult g = gmres(A, mg, B, S, rtol, restart, max_iters);
    std::memcpy(x, S.data(), N * sizeof(double));
    fill(g, out);
    return 0;
}

int ref_solve_bratu3d(size_t n, double lambda, int method, int precond_kind,
                      const numa_krylov_params* cp, const double* x0, double* x_out,
                      numa_krylov_result* res) {
    Bratu3D f(n, lambda);
    FdBratu op{f, cp ? cp->jvp_mode : 0, cp ? cp->d2_mode : 0};
    const KrylovParams p = to_params(cp);
    DVec X0(x0, x0 + f.size());
    KrylovResult r;
    if (precond_kind == NUMA_GPU_PRECOND_POISSON_MG) r = run(method, op, X0, p, PoissonMGProvider(n));
    else if (precond_kind == NUMA_GPU_PRECOND_JACOBI) r = run(method, op, X0, p, BratuJacobi{f});
    else r = run(method, op, X0, p, NoPrecond{});
    if (x_out) std::memcpy(x_out, r.x.data(), r.x.size() * sizeof(double));
    if (res) {
        std::memset(res, 0, sizeof(*res));
        res->converged = r.converged;
        res->iters = r.iters;
        res->n_F = r.n_F;
        res->n_JVP = r.n_JVP;
        res->n_D2 = r.n_D2;
        res->n_lin_iters = r.n_lin_iters;
        res->n_lin_failures = r.n_lin_failures;
        res->n_prec = r.n_prec;
        res->res0 = r.res0;
        res->res = r.res;
    }
    return 0;
}

double ref_forcing(const numa_krylov_params* cp, size_t k, double rnorm, double rprev,
                   double eta_prev, double res0) {
    return numa::op::detail::forcing(to_params(cp), k, rnorm, rprev, eta_prev, res0);
}

// ---- Burgers2D and HelmholtzMG2D (problems/burgers2d.hpp, linalg/helmholtz_mg2d.hpp)
int ref_burgers2d_exact(size_t n, double nu, double dt, double amp, double* out) {
    Burgers2D f(n, nu, dt, amp);
    std::memcpy(out, f.exact().data(), f.size() * sizeof(double));
    return 0;
}

int ref_burgers2d_eval(size_t n, double nu, double dt, double amp, const double* w, double* out) {
    Burgers2D f(n, nu, dt, amp);
    DVec W(w, w + f.size()), O;
    f.eval(W, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int ref_burgers2d_jvp(size_t n, double nu, double dt, double amp, const double* w, const double* d, double* out,
                      int mode) {
    Burgers2D f(n, nu, dt, amp);
    DVec W(w, w + f.size()), D(d, d + f.size()), O;
    if (mode == 1) jvp_fd(f, W, D, O); else f.jvp(W, D, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int ref_burgers2d_d2(size_t n, double nu, double dt, double amp, const double* w, const double* d, double* out,
                     int mode) {
    Burgers2D f(n, nu, dt, amp);
    DVec W(w, w + f.size()), D(d, d + f.size()), O;
    if (mode == 1) d2_fd(f, W, D, O); else f.d2(W, D, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int ref_hmg2d_levels(size_t n, double alpha, double nu) {
    HelmholtzMG2D mg(n, alpha, nu);
    return static_cast<int>(mg.levels());
}

int ref_hmg2d_apply(size_t n, double alpha, double nu, int pre, int post, const double* r, double* z) {
    HelmholtzMG2D mg(n, alpha, nu, pre, post);
    DVec R(r, r + n * n), Z;
    mg(R, Z);
    std::memcpy(z, Z.data(), Z.size() * sizeof(double));
    return 0;
}

namespace {
struct FdBurgers {
    const Burgers2D& f;
    int jvp_mode, d2_mode;
    std::size_t size() const { return f.size(); }
    void eval(const DVec& x, DVec& out) const { f.eval(x, out); }
    void jvp(const DVec& x, const DVec& v, DVec& out) const {
        if (jvp_mode == 1) jvp_fd(f, x, v, out); else f.jvp(x, v, out);
    }
    void d2(const DVec& x, const DVec& v, DVec& out) const {
        if (d2_mode == 1) d2_fd(f, x, v, out); else f.d2(x, v, out);
    }
};
}  // namespace

int ref_solve_burgers2d(size_t n, double nu, double dt, double amp, int method, int precond_kind,
                        const numa_krylov_params* cp, const double* x0, double* x_out, numa_krylov_result* res) {
    Burgers2D f(n, nu, dt, amp);
    FdBurgers op{f, cp ? cp->jvp_mode : 0, cp ? cp->d2_mode : 0};
    const KrylovParams p = to_params(cp);
    DVec X0(x0, x0 + f.size());
    KrylovResult r = precond_kind == NUMA_GPU_PRECOND_POISSON_MG ? run(method, op, X0, p, BurgersMGProvider(n, nu, dt))
                                                                 : run(method, op, X0, p, NoPrecond{});
    if (x_out) std::memcpy(x_out, r.x.data(), r.x.size() * sizeof(double));
    if (res) {
        std::memset(res, 0, sizeof(*res));
        res->converged = r.converged;
        res->iters = r.iters;
        res->n_F = r.n_F;
        res->n_JVP = r.n_JVP;
        res->n_D2 = r.n_D2;
        res->n_lin_iters = r.n_lin_iters;
        res->n_lin_failures = r.n_lin_failures;
        res->n_prec = r.n_prec;
        res->res0 = r.res0;
        res->res = r.res;
    }
    return 0;
}

// ---- Brusselator1DStep and BrusselatorJacobi (problems/brusselator1d.hpp)
int ref_bruss1d_previous(size_t n, double dt, double* out) {
    Brusselator1DStep f(n, dt);
    std::memcpy(out, f.previous().data(), f.size() * sizeof(double));
    return 0;
}

int ref_bruss1d_eval(size_t n, double dt, const double* w, double* out) {
    Brusselator1DStep f(n, dt);
    DVec W(w, w + f.size()), O;
    f.eval(W, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int ref_bruss1d_jvp(size_t n, double dt, const double* w, const double* d, double* out, int mode) {
    Brusselator1DStep f(n, dt);
    DVec W(w, w + f.size()), D(d, d + f.size()), O;
    if (mode == 1) jvp_fd(f, W, D, O); else f.jvp(W, D, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int ref_bruss1d_d2(size_t n, double dt, const double* w, const double* d, double* out, int mode) {
    Brusselator1DStep f(n, dt);
    DVec W(w, w + f.size()), D(d, d + f.size()), O;
    if (mode == 1) d2_fd(f, W, D, O); else f.d2(W, D, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int ref_bruss1d_jacobi_apply(size_t n, double dt, const double* w, const double* r, double* z) {
    Brusselator1DStep f(n, dt);
    BrusselatorJacobi pc{f};
    DVec W(w, w + f.size()), R(r, r + f.size()), Z;
    auto bound = pc.make(W);
    bound(R, Z);
    std::memcpy(z, Z.data(), Z.size() * sizeof(double));
    return 0;
}

namespace {
struct FdBruss {
    const Brusselator1DStep& f;
    int jvp_mode, d2_mode;
    std::size_t size() const { return f.size(); }
    void eval(const DVec& x, DVec& out) const { f.eval(x, out); }
    void jvp(const DVec& x, const DVec& v, DVec& out) const {
        if (jvp_mode == 1) jvp_fd(f, x, v, out); else f.jvp(x, v, out);
    }
    void d2(const DVec& x, const DVec& v, DVec& out) const {
        if (d2_mode == 1) d2_fd(f, x, v, out); else f.d2(x, v, out);
    }
};
}  // namespace

// From x0 (null: previous(), run_campaign.cpp's natural start) with NoPrecond or BrusselatorJacobi.
int ref_solve_bruss1d(size_t n, double dt, int method, int precond_kind, const numa_krylov_params* cp,
                      const double* x0, double* x_out, numa_krylov_result* res) {
    Brusselator1DStep f(n, dt);
    FdBruss op{f, cp ? cp->jvp_mode : 0, cp ? cp->d2_mode : 0};
    const KrylovParams p = to_params(cp);
    const DVec X0 = x0 ? DVec(x0, x0 + f.size()) : f.previous();
    KrylovResult r = precond_kind == NUMA_GPU_PRECOND_BRUSS_JACOBI ? run(method, op, X0, p, BrusselatorJacobi{f})
                                                                   : run(method, op, X0, p, NoPrecond{});
    if (x_out) std::memcpy(x_out, r.x.data(), r.x.size() * sizeof(double));
    if (res) {
        std::memset(res, 0, sizeof(*res));
        res->converged = r.converged;
        res->iters = r.iters;
        res->n_F = r.n_F;
        res->n_JVP = r.n_JVP;
        res->n_D2 = r.n_D2;
        res->n_lin_iters = r.n_lin_iters;
        res->n_lin_failures = r.n_lin_failures;
        res->n_prec = r.n_prec;
        res->res0 = r.res0;
        res->res = r.res;
    }
    return 0;
}

}  // extern "C"
