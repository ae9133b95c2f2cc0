// numa/gpu/numa_gpu.hpp — C++20 adaptor over the C ABI of libnuma_gpu.so (numa_gpu.h).
//
// The classes satisfy the reference's operator and preconditioner interfaces on
// std::vector<double> (operators/operator.hpp:43-58, krylov_newton.hpp:20-22), so code written
// against the reference — including its own templates gmres, newton_krylov, chebyshev_inexact —
// compiles unchanged against them; each such call moves its vectors to and from the GPU.  The
// DeviceVec overloads and the native drivers (newton_krylov / chebyshev_inexact /
// tf_chebyshev_2018 below) keep every vector on the GPU and are the fast path.
//
// Errors: a non-zero status from the library throws numa::gpu::Error; PoissonMG's size errors
// throw std::invalid_argument / std::overflow_error as the reference's constructor does
// (linalg/poisson_mg.hpp:29-42, :71-74).
#pragma once

#include <cstddef>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../numa_gpu.h"

namespace numa::gpu {

using DVec = std::vector<double>;

struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(int status, numa_gpu_ctx* ctx, const char* where) {
    if (status == NUMA_GPU_OK) return;
    std::string msg = std::string(where) + ": " + numa_gpu_status_string(status);
    if (ctx) {
        const char* d = numa_gpu_ctx_last_error(ctx);
        if (d && *d) msg += std::string(": ") + d;
    }
    if (status == NUMA_GPU_ERR_INVALID_ARGUMENT) throw std::invalid_argument(msg);
    if (status == NUMA_GPU_ERR_OVERFLOW) throw std::overflow_error(msg);
    throw Error(status, msg);
}

// One device and its stream.  Objects made on a context must be destroyed before it (declare the
// Context first: locals and members are destroyed in the reverse order).
class Context {
public:
    explicit Context(int device = 0) { check(numa_gpu_ctx_create(device, &h_), nullptr, "numa_gpu_ctx_create"); }
    ~Context() { numa_gpu_ctx_destroy(h_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    numa_gpu_ctx* get() const { return h_; }
    void synchronize() const { check(numa_gpu_ctx_synchronize(h_), h_, "synchronize"); }

private:
    numa_gpu_ctx* h_ = nullptr;
};

// A device FP64 vector (the reference's DVec, resident on the GPU).
class DeviceVec {
public:
    DeviceVec(const Context& ctx, std::size_t n) : ctx_(ctx.get()) {
        check(numa_gpu_vec_create(ctx_, n, &h_), ctx_, "numa_gpu_vec_create");
    }
    DeviceVec(const Context& ctx, const DVec& host) : DeviceVec(ctx, host.size()) { upload(host); }
    ~DeviceVec() { numa_gpu_vec_destroy(h_); }
    DeviceVec(const DeviceVec&) = delete;
    DeviceVec& operator=(const DeviceVec&) = delete;
    DeviceVec(DeviceVec&& o) noexcept : ctx_(o.ctx_), h_(std::exchange(o.h_, nullptr)) {}
    std::size_t size() const {
        std::size_t n = 0;
        numa_gpu_vec_size(h_, &n);
        return n;
    }
    void upload(const DVec& host) { check(numa_gpu_vec_upload(h_, host.data(), host.size()), ctx_, "upload"); }
    void download(DVec& host) const {
        host.resize(size());
        check(numa_gpu_vec_download(h_, host.data(), host.size()), ctx_, "download");
    }
    DVec to_host() const {
        DVec v;
        download(v);
        return v;
    }
    numa_gpu_vec* get() const { return h_; }

private:
    numa_gpu_ctx* ctx_;
    numa_gpu_vec* h_ = nullptr;
};

inline double dot(const DeviceVec& a, const DeviceVec& b) {
    double s = 0;
    check(numa_gpu_vec_dot(a.get(), b.get(), &s), nullptr, "dot");
    return s;
}
inline double norm2(const DeviceVec& a) {
    double s = 0;
    check(numa_gpu_vec_norm2(a.get(), &s), nullptr, "norm2");
    return s;
}
inline void axpy(double a, const DeviceVec& x, DeviceVec& y) { check(numa_gpu_vec_axpy(a, x.get(), y.get()), nullptr, "axpy"); }

// Bratu3D(n, lambda) (problems/bratu3d.hpp:12-100): NonlinearOperator and SecondOrderOperator.
class Bratu3D {
public:
    Bratu3D(const Context& ctx, std::size_t n, double lambda = 1.0) : ctx_(&ctx), n_(n) {
        check(numa_gpu_bratu3d_create(ctx.get(), n, lambda, &h_), ctx.get(), "numa_gpu_bratu3d_create");
    }
    ~Bratu3D() { numa_gpu_bratu3d_destroy(h_); }
    Bratu3D(const Bratu3D&) = delete;
    Bratu3D& operator=(const Bratu3D&) = delete;

    std::size_t size() const { return n_ * n_ * n_; }
    std::size_t grid() const { return n_; }
    numa_gpu_bratu3d* get() const { return h_; }
    const Context& context() const { return *ctx_; }

    // device-vector forms
    void eval(const DeviceVec& x, DeviceVec& out) const {
        check(numa_gpu_bratu3d_eval(h_, x.get(), out.get()), ctx_->get(), "eval");
    }
    void jvp(const DeviceVec& x, const DeviceVec& v, DeviceVec& out, int mode = NUMA_GPU_DERIV_ANALYTIC) const {
        check(numa_gpu_bratu3d_jvp(h_, x.get(), v.get(), out.get(), mode), ctx_->get(), "jvp");
    }
    void d2(const DeviceVec& x, const DeviceVec& v, DeviceVec& out, int mode = NUMA_GPU_DERIV_ANALYTIC) const {
        check(numa_gpu_bratu3d_d2(h_, x.get(), v.get(), out.get(), mode), ctx_->get(), "d2");
    }
    void jacobi_diag(const DeviceVec& x, DeviceVec& d) const {
        check(numa_gpu_bratu3d_jacobi_diag(h_, x.get(), d.get()), ctx_->get(), "jacobi_diag");
    }

    // host-vector forms (the reference concepts): upload, compute, download
    void eval(const DVec& x, DVec& out) const {
        DeviceVec dx(*ctx_, x), dout(*ctx_, size());
        eval(dx, dout);
        dout.download(out);
    }
    void jvp(const DVec& x, const DVec& v, DVec& out) const {
        DeviceVec dx(*ctx_, x), dv(*ctx_, v), dout(*ctx_, size());
        jvp(dx, dv, dout);
        dout.download(out);
    }
    void d2(const DVec& x, const DVec& v, DVec& out) const {
        DeviceVec dx(*ctx_, x), dv(*ctx_, v), dout(*ctx_, size());
        d2(dx, dv, dout);
        dout.download(out);
    }
    void jacobi_diag(const DVec& x, DVec& d) const {
        DeviceVec dx(*ctx_, x), dd(*ctx_, size());
        jacobi_diag(dx, dd);
        dd.download(d);
    }

private:
    const Context* ctx_;
    std::size_t n_;
    numa_gpu_bratu3d* h_ = nullptr;
};

// PoissonMG(n, pre, post) (linalg/poisson_mg.hpp:24-299): callable as a preconditioner (r, z).
class PoissonMG {
public:
    PoissonMG(const Context& ctx, std::size_t n, int pre = 2, int post = 2, int precision = NUMA_GPU_FP64)
        : ctx_(&ctx), n_(n) {
        check(numa_gpu_mg_create_ex(ctx.get(), n, pre, post, precision, 0, &h_), ctx.get(), "PoissonMG");
    }
    ~PoissonMG() { numa_gpu_mg_destroy(h_); }
    PoissonMG(const PoissonMG&) = delete;
    PoissonMG& operator=(const PoissonMG&) = delete;
    std::size_t levels() const {
        std::size_t l = 0;
        numa_gpu_mg_levels(h_, &l);
        return l;
    }
    void operator()(const DeviceVec& r, DeviceVec& z) const { check(numa_gpu_mg_apply(h_, r.get(), z.get()), ctx_->get(), "PoissonMG"); }
    void operator()(const DVec& r, DVec& z) const {
        DeviceVec dr(*ctx_, r), dz(*ctx_, r.size());
        (*this)(dr, dz);
        dz.download(z);
    }

private:
    const Context* ctx_;
    std::size_t n_;
    numa_gpu_mg* h_ = nullptr;
};

// Preconditioner providers: make(x) -> Bound, Bound(r, z) (krylov_newton.hpp:20-22).
class Provider {
public:
    ~Provider() { numa_gpu_provider_destroy(h_); }
    Provider(const Provider&) = delete;
    Provider& operator=(const Provider&) = delete;
    Provider(Provider&& o) noexcept : ctx_(o.ctx_), h_(std::exchange(o.h_, nullptr)) {}

    static Provider identity(const Context& ctx) {
        numa_gpu_provider* h = nullptr;
        check(numa_gpu_provider_create_identity(ctx.get(), &h), ctx.get(), "NoPrecond");
        return Provider(ctx, h);
    }
    static Provider poisson_mg(const Context& ctx, std::size_t n, int precision = NUMA_GPU_FP64) {
        numa_gpu_provider* h = nullptr;
        check(numa_gpu_provider_create_poisson_mg(ctx.get(), n, 2, 2, precision, &h), ctx.get(), "PoissonMGProvider");
        return Provider(ctx, h);
    }
    // Extension: the FP32 V-cycle whose levels n <= 15 solve with the Jacobian -Lap_h - lambda e^u of the
    // iterate it is made at (numa_gpu_provider_create_jacobian_mg; with flexible = 1, jvp_precision = FP32
    // and jvp_tight = 1 in the parameters, the benchmark's mixed path).
    static Provider jacobian_mg(const Context& ctx, std::size_t n) {
        numa_gpu_provider* h = nullptr;
        check(numa_gpu_provider_create_jacobian_mg(ctx.get(), n, 2, 2, &h), ctx.get(), "JacobianMGProvider");
        return Provider(ctx, h);
    }
    static Provider jacobi(const Bratu3D& f) {
        numa_gpu_provider* h = nullptr;
        check(numa_gpu_provider_create_jacobi(f.get(), &h), f.context().get(), "BratuJacobi");
        return Provider(f.context(), h);
    }

    struct Bound {
        const Provider* p;
        void operator()(const DeviceVec& r, DeviceVec& z) const {
            check(numa_gpu_provider_apply(p->h_, r.get(), z.get()), p->ctx_->get(), "precond");
        }
        void operator()(const DVec& r, DVec& z) const {
            DeviceVec dr(*p->ctx_, r), dz(*p->ctx_, r.size());
            (*this)(dr, dz);
            dz.download(z);
        }
    };
    Bound make(const DeviceVec& x) const {
        check(numa_gpu_provider_make(h_, x.get()), ctx_->get(), "make");
        return Bound{this};
    }
    Bound make(const DVec& x) const {
        DeviceVec dx(*ctx_, x);
        return make(dx);
    }
    numa_gpu_provider* get() const { return h_; }

private:
    Provider(const Context& ctx, numa_gpu_provider* h) : ctx_(&ctx), h_(h) {}
    const Context* ctx_;
    numa_gpu_provider* h_ = nullptr;
};

// KrylovParams / KrylovResult with the reference's field names (krylov_newton.hpp:24-49).
struct KrylovParams : numa_krylov_params {
    KrylovParams() { numa_krylov_params_default(this); }
};

struct KrylovResult {
    DVec x;
    bool converged = false;
    std::size_t iters = 0;
    std::size_t n_F = 0, n_JVP = 0, n_D2 = 0;
    std::size_t n_lin_iters = 0;
    std::size_t n_lin_failures = 0;
    std::size_t n_prec = 0;
    double res0 = 0.0, res = 0.0;
    numa_krylov_result raw{};  // plus per-primitive timers
};

namespace detail {
inline KrylovResult run(int method, const Bratu3D& f, DVec x, const KrylovParams& p, const Provider* pc) {
    DeviceVec dx(f.context(), x);
    numa_krylov_result r{};
    numa_gpu_provider* ph = pc ? pc->get() : nullptr;
    int s;
    if (method == NUMA_GPU_METHOD_NK) s = numa_gpu_newton_krylov(f.get(), dx.get(), &p, ph, &r);
    else if (method == NUMA_GPU_METHOD_TF2018) s = numa_gpu_tf_chebyshev_2018(f.get(), dx.get(), &p, ph, &r);
    else {
        KrylovParams q = p;
        if (method == NUMA_GPU_METHOD_CHEB_REC) q.recycle = 1;
        s = numa_gpu_chebyshev_inexact(f.get(), dx.get(), &q, ph, &r);
    }
    check(s, f.context().get(), "nonlinear solve");
    KrylovResult out;
    dx.download(out.x);
    out.converged = r.converged != 0;
    out.iters = r.iters;
    out.n_F = r.n_F;
    out.n_JVP = r.n_JVP;
    out.n_D2 = r.n_D2;
    out.n_lin_iters = r.n_lin_iters;
    out.n_lin_failures = r.n_lin_failures;
    out.n_prec = r.n_prec;
    out.res0 = r.res0;
    out.res = r.res;
    out.raw = r;
    return out;
}
}  // namespace detail

// Native drivers: the reference's signatures (krylov_newton.hpp:69-71, :116-118,
// tf_chebyshev_2018.hpp:52-57) with every vector on the GPU during the solve.
inline KrylovResult newton_krylov(const Bratu3D& f, DVec x, const KrylovParams& p = {}, const Provider* pc = nullptr) {
    return detail::run(NUMA_GPU_METHOD_NK, f, std::move(x), p, pc);
}
inline KrylovResult chebyshev_inexact(const Bratu3D& f, DVec x, const KrylovParams& p = {},
                                      const Provider* pc = nullptr) {
    return detail::run(NUMA_GPU_METHOD_CHEB, f, std::move(x), p, pc);
}
inline KrylovResult tf_chebyshev_2018(const Bratu3D& f, DVec x, const KrylovParams& p = {},
                                      const Provider* pc = nullptr) {
    return detail::run(NUMA_GPU_METHOD_TF2018, f, std::move(x), p, pc);
}

}  // namespace numa::gpu
