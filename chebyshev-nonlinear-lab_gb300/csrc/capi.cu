// capi.cu — the extern "C" boundary of libnuma_gpu.so (declared in include/numa_gpu.h).
//
// Every entry point validates its handles and sizes, runs the C++ implementation and converts
// exceptions into status codes (the reference reports failure through result structs and, for
// PoissonMG, std::invalid_argument / std::overflow_error: those map to
// NUMA_GPU_ERR_INVALID_ARGUMENT / NUMA_GPU_ERR_OVERFLOW).
#include <cstring>
#include <mutex>
#include <memory>
#include <new>
#include <string>

#include "numa_internal.hpp"

using namespace numa::gpu;

struct numa_gpu_bratu3d {
    numa_gpu_ctx* ctx;
    std::unique_ptr<Bratu3D> impl;
};
struct numa_gpu_mg {
    numa_gpu_ctx* ctx;
    std::unique_ptr<PoissonMG> impl;
};
struct numa_gpu_provider {
    numa_gpu_ctx* ctx;
    std::unique_ptr<Provider> impl;
    size_t N;  // 0 = any size (identity)
};
struct numa_gpu_krylov_space {
    numa_gpu_ctx* ctx;
    KrylovSpace impl;
};
struct numa_gpu_burgers2d {
    numa_gpu_ctx* ctx;
    std::unique_ptr<Burgers2D> impl;
};
struct numa_gpu_learned {
    numa_gpu_ctx* ctx;
    LearnedNet* impl;
    ~numa_gpu_learned() { learned_destroy(impl); }
};
struct numa_gpu_hmg2d {
    numa_gpu_ctx* ctx;
    std::unique_ptr<HelmholtzMG2D> impl;
};
struct numa_gpu_brusselator1d {
    numa_gpu_ctx* ctx;
    std::unique_ptr<Brusselator1D> impl;
};
struct numa_gpu_brusselator2d {
    numa_gpu_ctx* ctx;
    std::unique_ptr<Brusselator2D> impl;
};
struct numa_gpu_bmg2d {
    numa_gpu_ctx* ctx;
    std::unique_ptr<BrussMG2D> impl;
};

namespace {

// Per-context caches owned by the C layer.
struct CtxExtras {
    std::unique_ptr<Gmres> gmres;
    size_t gmres_N = 0;
    // numa_gpu_solve_bratu3d_host keeps its operator, provider and vector between calls
    std::unique_ptr<Bratu3D> host_op;
    std::unique_ptr<Provider> host_pc;
    DeviceArray<double> host_x;
    std::unique_ptr<HostUpload> host_up;  // the staged upload of a pinned x0 (Newton–Krylov)
    size_t host_n = 0;
    double host_lambda = 0.0;
    int host_kind = -1, host_prec = -1;
    // numa_gpu_solve_burgers2d_host likewise
    std::unique_ptr<Burgers2D> bh_op;
    std::unique_ptr<Provider> bh_pc;
    DeviceArray<double> bh_x;
    size_t bh_n = 0;
    double bh_nu = 0.0, bh_dt = 0.0, bh_amp = 0.0;
    int bh_kind = -1;
    // numa_gpu_brusselator2d_advance_host likewise
    std::unique_ptr<Brusselator2D> b2_op;
    std::unique_ptr<Provider> b2_pc;
    DeviceArray<double> b2_x;
    size_t b2_n = 0;
    numa_brusselator2d_params b2_p{};
    int b2_kind = -1, b2_prec = -1;
};

struct CtxHandle : numa_gpu_ctx {
    std::unique_ptr<Context> own;
    CtxExtras extras;
};

CtxExtras& extras(numa_gpu_ctx* c) { return static_cast<CtxHandle*>(c)->extras; }

template <class F>
int guard(numa_gpu_ctx* ctx, F&& fn) {
    try {
        fn();
        if (ctx && ctx->impl) ctx->impl->last_error.clear();
        return NUMA_GPU_OK;
    } catch (const Status& s) {
        if (ctx && ctx->impl) ctx->impl->last_error = s.what();
        return s.code;
    } catch (const std::bad_alloc&) {
        if (ctx && ctx->impl) ctx->impl->last_error = "host allocation failed";
        return NUMA_GPU_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        if (ctx && ctx->impl) ctx->impl->last_error = e.what();
        return NUMA_GPU_ERR_CUDA;
    }
}

void need(bool cond, int code, const char* msg) {
    if (!cond) throw Status(code, msg);
}

void same_ctx(numa_gpu_ctx* a, const numa_gpu_vec* v) {
    need(v != nullptr, NUMA_GPU_ERR_INVALID_ARGUMENT, "null vector");
    need(v->ctx == a, NUMA_GPU_ERR_INVALID_ARGUMENT, "vector belongs to another context");
}

void sized(const numa_gpu_vec* v, size_t N) {
    need(v->n == N, NUMA_GPU_ERR_SIZE_MISMATCH, "vector length does not match the operator size");
}

Gmres& gmres_for(numa_gpu_ctx* c, size_t N) {
    CtxExtras& e = extras(c);
    if (!e.gmres || e.gmres_N != N) {
        e.gmres = std::make_unique<Gmres>(*c->impl, N);
        e.gmres_N = N;
    }
    return *e.gmres;
}

// C callbacks as LinearOp / Precond over non-owning vector views.
struct CallbackOp : LinearOp {
    numa_gpu_ctx* ctx;
    numa_gpu_apply_fn fn;
    void* user;
    size_t N;
    void apply(const double* v, double* out) override {
        numa_gpu_vec vv{ctx, const_cast<double*>(v), N, false}, ov{ctx, out, N, false};
        if (fn(user, &vv, &ov) != 0) throw Status(NUMA_GPU_ERR_CALLBACK, "apply callback returned an error");
    }
};
struct CallbackPrec : Precond {
    numa_gpu_ctx* ctx;
    numa_gpu_precond_fn fn;
    void* user;
    size_t N;
    void apply(const double* r, double* z) override {
        numa_gpu_vec rv{ctx, const_cast<double*>(r), N, false}, zv{ctx, z, N, false};
        if (fn(user, &rv, &zv) != 0) throw Status(NUMA_GPU_ERR_CALLBACK, "precond callback returned an error");
    }
};

// Jacobian of a Bratu3D at a fixed point.
// The Bratu3D Jacobian at a point as a linear operator: analytic (FP64), analytic in FP32 arithmetic
// (bound as the mixed drivers bind it, with the FP32 product forms FGMRES uses), or by finite
// differences.
struct BratuJacOp : LinearOp {
    Bratu3D& f;
    int mode;
    const double *x, *c, *fx, *xnorm;
    BratuJacOp(Bratu3D& f_, int m) : f(f_), mode(m), x(nullptr), c(nullptr), fx(nullptr), xnorm(nullptr) {}
    ~BratuJacOp() override {
        if (mode == NUMA_GPU_DERIV_ANALYTIC_FP32) f.prepare_cache(NUMA_GPU_FP64);
    }
    void apply(const double* v, double* out) override {
        if (mode == NUMA_GPU_DERIV_FD) f.jvp_fd(x, fx, xnorm, v, out);
        else if (mode == NUMA_GPU_DERIV_ANALYTIC_FP32) f.jvp_bound(v, out);
        else f.jvp_c(c, v, out);
    }
    bool has_apply32() const override { return mode == NUMA_GPU_DERIV_ANALYTIC_FP32 && f.has_jvp32(); }
    void apply32(const float* v32, double* out) override { f.jvp_bound32(v32, out); }
    bool has_apply32f() const override { return mode == NUMA_GPU_DERIV_ANALYTIC_FP32 && f.has_jvp32f(); }
    void apply32f(const float* v32, float* out32) override { f.jvp_bound32f(v32, out32); }
};
struct ProviderPrec : Precond {
    Provider* p;
    void apply(const double* r, double* z) override { p->apply(r, z); }
    bool has_apply32() const override { return p->has_apply32(); }
    void apply32(const double* r, float* z32) override { p->apply32(r, z32); }
    bool has_apply32f() const override { return p->has_apply32f(); }
    void apply32f(const float* r32, float* z32) override { p->apply32f(r32, z32); }
};

// Checks a driver's vector and provider against an operator of size N.
void check_driver_args(numa_gpu_ctx* ctx, const numa_gpu_vec* x, size_t N, const numa_gpu_provider* provider) {
    same_ctx(ctx, x);
    sized(x, N);
    if (provider) {
        need(provider->ctx == ctx, NUMA_GPU_ERR_INVALID_ARGUMENT, "provider belongs to another context");
        need(provider->N == 0 || provider->N == N, NUMA_GPU_ERR_SIZE_MISMATCH, "provider size differs");
    }
}

// method of numa_gpu_method on any operator (the reference's templated drivers).
void dispatch_driver(int method, NonlinearOp& f, double* x, const numa_krylov_params* p, Provider* pc,
                     numa_krylov_result& out) {
    need(method >= NUMA_GPU_METHOD_NK && method <= NUMA_GPU_METHOD_TF2018, NUMA_GPU_ERR_INVALID_ARGUMENT,
         "unknown method");
    KrylovParams kp = params_from_c(p);
    if (method == NUMA_GPU_METHOD_NK) newton_krylov(f, x, kp, pc, out);
    else if (method == NUMA_GPU_METHOD_TF2018) tf_chebyshev_2018(f, x, kp, pc, out);
    else {
        if (method == NUMA_GPU_METHOD_CHEB_REC) kp.recycle = true;
        chebyshev_inexact(f, x, kp, pc, out);
    }
}

// out = F'(x) v or F''(x)[v, v] of any operator, analytic or by finite differences, for the
// per-operator entry points (temporaries are freed on return, hence the synchronisation).
void op_derivative(NonlinearOp& f, bool second, const double* x, const double* v, double* out, int mode) {
    Context& c = f.ctx();
    const size_t N = f.size();
    if (mode == NUMA_GPU_DERIV_FD) {
        DeviceArray<double> f0(N);
        f.eval(x, f0.p, nullptr, nullptr);
        dev_norm2(c, x, N, c.scalar(kSlotTmp1));
        if (second) f.d2_fd(x, f0.p, c.scalar(kSlotTmp1), v, out);
        else f.jvp_fd(x, f0.p, c.scalar(kSlotTmp1), v, out);
        c.sync();
        return;
    }
    need(mode == NUMA_GPU_DERIV_ANALYTIC || (mode == NUMA_GPU_DERIV_ANALYTIC_FP32 && !second),
         NUMA_GPU_ERR_INVALID_ARGUMENT, "unknown derivative mode");
    if (mode == NUMA_GPU_DERIV_ANALYTIC_FP32) {
        // the product the drivers use with jvp_precision = FP32 (FP64 where an operator has no FP32 form)
        f.prepare_cache(NUMA_GPU_FP32);  // before sizing: the FP32 form may keep more in the cache
        DeviceArray<double> cache(f.cache_size());
        DeviceArray<double> tmp(f.cache_size() ? N : 0);
        if (f.cache_size()) f.eval(x, tmp.p, cache.p, nullptr);
        f.bind(x, cache.p, NUMA_GPU_FP32);
        f.jvp_bound(v, out);
        f.prepare_cache(NUMA_GPU_FP64);
        c.sync();
        return;
    }
    if (!second) {
        f.jvp_at(x, v, out);
        return;
    }
    DeviceArray<double> cache(f.cache_size());
    DeviceArray<double> tmp(f.cache_size() ? N : 0);
    if (f.cache_size()) f.eval(x, tmp.p, cache.p, nullptr);
    f.d2(x, cache.p, v, out);
    c.sync();
}

void fill_gmres(const GmresResult& g, numa_gmres_result* out) {
    if (!out) return;
    out->iters = g.iters;
    out->matvecs = g.matvecs;
    out->precs = g.precs;
    out->rel_res = g.rel_res;
    out->converged = g.converged ? 1 : 0;
    out->breakdown = g.breakdown ? 1 : 0;
}

GmresOptions gopts(double rtol, size_t restart, size_t max_iters, int zero_guess, int orth, int flexible) {
    GmresOptions o;
    o.rtol = rtol;
    o.restart = restart;
    o.max_iters = max_iters;
    o.zero_guess = zero_guess != 0;
    o.orth = orth;
    o.flexible = flexible != 0;
    return o;
}

}  // namespace

extern "C" {

int numa_gpu_abi_version(void) { return NUMA_GPU_ABI_VERSION; }

const char* numa_gpu_status_string(int s) {
    switch (s) {
        case NUMA_GPU_OK: return "ok";
        case NUMA_GPU_ERR_INVALID_ARGUMENT: return "invalid argument";
        case NUMA_GPU_ERR_OVERFLOW: return "size overflow";
        case NUMA_GPU_ERR_SIZE_MISMATCH: return "size mismatch";
        case NUMA_GPU_ERR_CUDA: return "CUDA error";
        case NUMA_GPU_ERR_OUT_OF_MEMORY: return "out of memory";
        case NUMA_GPU_ERR_NO_DEVICE: return "no CUDA device";
        case NUMA_GPU_ERR_CALLBACK: return "callback error";
        case NUMA_GPU_ERR_NOT_SUPPORTED: return "not supported";
        case NUMA_GPU_ERR_TOO_LARGE: return "too large for the fixed scratch array";
        default: return "unknown status";
    }
}

void numa_krylov_params_default(numa_krylov_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->rtol_nl = 1e-8;
    p->max_nl = 50;
    p->eta_init = 0.5;
    p->eta_max = 0.9;
    p->gamma = 0.9;
    p->alpha = 2.0;
    p->eta2_factor = 10.0;
    p->eta2_max = 0.5;
    p->gmres_restart = 50;
    p->gmres_max_iters = 500;
    p->armijo = 1e-4;
    p->min_lambda = 1e-4;
}

// ------------------------------------------------------------------------------ context
int numa_gpu_ctx_create(int device, numa_gpu_ctx** out) {
    if (!out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    try {
        auto h = std::make_unique<CtxHandle>();
        h->own = std::make_unique<Context>(device);
        h->impl = h->own.get();
        *out = h.release();
        return NUMA_GPU_OK;
    } catch (const Status& s) {
        return s.code;
    } catch (const std::bad_alloc&) {
        return NUMA_GPU_ERR_OUT_OF_MEMORY;
    } catch (...) {
        return NUMA_GPU_ERR_CUDA;
    }
}

int numa_gpu_ctx_destroy(numa_gpu_ctx* ctx) {
    if (!ctx) return NUMA_GPU_OK;
    CtxHandle* h = static_cast<CtxHandle*>(ctx);
    h->extras = CtxExtras();
    delete h;
    return NUMA_GPU_OK;
}

int numa_gpu_ctx_synchronize(numa_gpu_ctx* ctx) {
    if (!ctx) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(ctx, [&] { ctx->impl->sync(); });
}

const char* numa_gpu_ctx_last_error(numa_gpu_ctx* ctx) {
    if (!ctx || !ctx->impl) return "";
    return ctx->impl->last_error.c_str();
}

int numa_gpu_ctx_set_timing(numa_gpu_ctx* ctx, int enable) {
    if (!ctx) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    ctx->impl->timing = enable != 0;
    return NUMA_GPU_OK;
}

int numa_gpu_ctx_kernel_launches(numa_gpu_ctx* ctx, uint64_t* out) {
    if (!ctx || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = ctx->impl->launches;
    return NUMA_GPU_OK;
}

int numa_gpu_ctx_reset_kernel_launches(numa_gpu_ctx* ctx) {
    if (!ctx) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    ctx->impl->launches = 0;
    return NUMA_GPU_OK;
}

int numa_gpu_ctx_stream(numa_gpu_ctx* ctx, void** stream_out) {
    if (!ctx || !stream_out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *stream_out = reinterpret_cast<void*>(ctx->impl->stream);
    return NUMA_GPU_OK;
}

// ------------------------------------------------------------------------------ vectors
int numa_gpu_vec_create(numa_gpu_ctx* ctx, size_t n, numa_gpu_vec** out) {
    if (!ctx || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto v = std::make_unique<numa_gpu_vec>();
        v->ctx = ctx;
        v->n = n;
        v->owns = true;
        v->d = nullptr;
        if (n > 0) {
            std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
            cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&v->d), n * sizeof(double));
            if (e == cudaErrorMemoryAllocation) {
                cudaGetLastError();
                throw Status(NUMA_GPU_ERR_OUT_OF_MEMORY, "cudaMalloc failed for a vector");
            }
            NUMA_CUDA(e);
            NUMA_CUDA(cudaMemsetAsync(v->d, 0, n * sizeof(double), ctx->impl->stream));
        }
        *out = v.release();
    });
}

int numa_gpu_vec_destroy(numa_gpu_vec* v) {
    if (!v) return NUMA_GPU_OK;
    if (v->owns && v->d) {
        cudaStreamSynchronize(v->ctx->impl->stream);
        std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
        cudaFree(v->d);
    }
    delete v;
    return NUMA_GPU_OK;
}

int numa_gpu_vec_size(const numa_gpu_vec* v, size_t* n) {
    if (!v || !n) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *n = v->n;
    return NUMA_GPU_OK;
}

int numa_gpu_vec_device_ptr(numa_gpu_vec* v, double** dptr) {
    if (!v || !dptr) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *dptr = v->d;
    return NUMA_GPU_OK;
}

int numa_gpu_vec_upload(numa_gpu_vec* v, const double* host, size_t n) {
    if (!v || (!host && n)) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(v->ctx, [&] {
        need(n == v->n, NUMA_GPU_ERR_SIZE_MISMATCH, "upload length differs from the vector length");
        if (n) NUMA_CUDA(cudaMemcpyAsync(v->d, host, n * sizeof(double), cudaMemcpyHostToDevice, v->ctx->impl->stream));
        v->ctx->impl->sync();
    });
}

int numa_gpu_vec_download(const numa_gpu_vec* v, double* host, size_t n) {
    if (!v || (!host && n)) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(v->ctx, [&] {
        need(n == v->n, NUMA_GPU_ERR_SIZE_MISMATCH, "download length differs from the vector length");
        if (n) NUMA_CUDA(cudaMemcpyAsync(host, v->d, n * sizeof(double), cudaMemcpyDeviceToHost, v->ctx->impl->stream));
        v->ctx->impl->sync();
    });
}

int numa_gpu_vec_fill(numa_gpu_vec* v, double value) {
    if (!v) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(v->ctx, [&] { dev_fill(*v->ctx->impl, v->d, value, v->n); });
}

int numa_gpu_vec_copy(const numa_gpu_vec* src, numa_gpu_vec* dst) {
    if (!src || !dst) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(dst->ctx, [&] {
        same_ctx(dst->ctx, src);
        need(src->n == dst->n, NUMA_GPU_ERR_SIZE_MISMATCH, "copy between vectors of different lengths");
        dev_copy(*dst->ctx->impl, src->d, dst->d, src->n);
    });
}

int numa_gpu_vec_dot(const numa_gpu_vec* a, const numa_gpu_vec* b, double* out) {
    if (!a || !b || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(a->ctx, [&] {
        same_ctx(a->ctx, b);
        need(a->n == b->n, NUMA_GPU_ERR_SIZE_MISMATCH, "dot of vectors of different lengths");
        Context& c = *a->ctx->impl;
        if (a->n == 0) {
            *out = 0.0;
            return;
        }
        dev_dot(c, a->d, b->d, a->n, c.scalar(kSlotTmp0));
        *out = c.fetch1(c.scalar(kSlotTmp0));
    });
}

int numa_gpu_vec_norm2(const numa_gpu_vec* a, double* out) {
    if (!a || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(a->ctx, [&] {
        Context& c = *a->ctx->impl;
        if (a->n == 0) {
            *out = 0.0;
            return;
        }
        dev_norm2(c, a->d, a->n, c.scalar(kSlotTmp0));
        *out = c.fetch1(c.scalar(kSlotTmp0));
    });
}

int numa_gpu_vec_axpy(double a, const numa_gpu_vec* x, numa_gpu_vec* y) {
    if (!x || !y) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(y->ctx, [&] {
        same_ctx(y->ctx, x);
        need(x->n == y->n, NUMA_GPU_ERR_SIZE_MISMATCH, "axpy of vectors of different lengths");
        dev_axpy(*y->ctx->impl, a, x->d, y->d, x->n);
    });
}

// ------------------------------------------------------------------------------ Bratu3D
int numa_gpu_bratu3d_create(numa_gpu_ctx* ctx, size_t n, double lambda, numa_gpu_bratu3d** out) {
    if (!ctx || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        need(n > 0, NUMA_GPU_ERR_INVALID_ARGUMENT, "Bratu3D needs n > 0");
        need(n <= 65535, NUMA_GPU_ERR_OVERFLOW, "Bratu3D grid too large");
        auto h = std::make_unique<numa_gpu_bratu3d>();
        h->ctx = ctx;
        h->impl = std::make_unique<Bratu3D>(*ctx->impl, n, lambda);
        *out = h.release();
    });
}

int numa_gpu_bratu3d_destroy(numa_gpu_bratu3d* op) {
    if (op) {
        cudaStreamSynchronize(op->ctx->impl->stream);
        delete op;
    }
    return NUMA_GPU_OK;
}

int numa_gpu_bratu3d_size(const numa_gpu_bratu3d* op, size_t* N) {
    if (!op || !N) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *N = op->impl->size();
    return NUMA_GPU_OK;
}

int numa_gpu_bratu3d_eval(numa_gpu_bratu3d* op, const numa_gpu_vec* x, numa_gpu_vec* out) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(op->ctx, [&] {
        same_ctx(op->ctx, x);
        same_ctx(op->ctx, out);
        sized(x, op->impl->size());
        sized(out, op->impl->size());
        need(x->d != out->d, NUMA_GPU_ERR_INVALID_ARGUMENT, "eval input and output must differ");
        op->impl->eval(x->d, out->d);
    });
}

int numa_gpu_bratu3d_jvp(numa_gpu_bratu3d* op, const numa_gpu_vec* x, const numa_gpu_vec* v, numa_gpu_vec* out,
                         int mode) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(op->ctx, [&] {
        for (const numa_gpu_vec* q : {x, v, (const numa_gpu_vec*)out}) {
            same_ctx(op->ctx, q);
            sized(q, op->impl->size());
        }
        need(out->d != x->d && out->d != v->d, NUMA_GPU_ERR_INVALID_ARGUMENT, "jvp output must not alias an input");
        Bratu3D& f = *op->impl;
        Context& c = *op->ctx->impl;
        if (mode == NUMA_GPU_DERIV_FD) {
            DeviceArray<double> f0(f.size());
            f.eval(x->d, f0.p);
            dev_norm2(c, x->d, f.size(), c.scalar(kSlotTmp1));
            f.jvp_fd(x->d, f0.p, c.scalar(kSlotTmp1), v->d, out->d);
            c.sync();
        } else if (mode == NUMA_GPU_DERIV_ANALYTIC_FP32) {
            DeviceArray<double> c64(f.size());
            DeviceArray<float> c32(f.size());
            f.coef(x->d, c64.p);
            f.coef32(c64.p, c32.p);
            f.jvp_c32(c32.p, v->d, out->d);
            c.sync();  // the temporaries are freed on return
        } else if (mode == NUMA_GPU_DERIV_ANALYTIC_FP32X) {
            DeviceArray<double> c64(f.size());
            DeviceArray<float> v32(f.size());
            f.coef(x->d, c64.p);
            f.coef32(v->d, v32.p);  // RN32(v): the same integer conversion as RN32(c)
            f.jvp_c32x(c64.p, v32.p, out->d);
            c.sync();
        } else {
            need(mode == NUMA_GPU_DERIV_ANALYTIC, NUMA_GPU_ERR_INVALID_ARGUMENT, "unknown derivative mode");
            f.jvp_x(x->d, v->d, out->d);
        }
    });
}

int numa_gpu_bratu3d_d2(numa_gpu_bratu3d* op, const numa_gpu_vec* x, const numa_gpu_vec* v, numa_gpu_vec* out,
                        int mode) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(op->ctx, [&] {
        for (const numa_gpu_vec* q : {x, v, (const numa_gpu_vec*)out}) {
            same_ctx(op->ctx, q);
            sized(q, op->impl->size());
        }
        need(out->d != x->d && out->d != v->d, NUMA_GPU_ERR_INVALID_ARGUMENT, "d2 output must not alias an input");
        Bratu3D& f = *op->impl;
        Context& c = *op->ctx->impl;
        DeviceArray<double> tmp(f.size());
        if (mode == NUMA_GPU_DERIV_FD) {
            f.eval(x->d, tmp.p);
            dev_norm2(c, x->d, f.size(), c.scalar(kSlotTmp1));
            f.d2_fd(x->d, tmp.p, c.scalar(kSlotTmp1), v->d, out->d);
        } else {
            need(mode == NUMA_GPU_DERIV_ANALYTIC, NUMA_GPU_ERR_INVALID_ARGUMENT, "unknown derivative mode");
            f.coef(x->d, tmp.p);
            f.d2_c(tmp.p, v->d, out->d);
        }
        c.sync();
    });
}

int numa_gpu_bratu3d_jacobi_diag(numa_gpu_bratu3d* op, const numa_gpu_vec* x, numa_gpu_vec* d) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(op->ctx, [&] {
        same_ctx(op->ctx, x);
        same_ctx(op->ctx, d);
        sized(x, op->impl->size());
        sized(d, op->impl->size());
        if (x->d == d->d) {
            DeviceArray<double> tmp(op->impl->size());
            op->impl->coef(x->d, tmp.p);
            op->impl->jacobi_diag_c(tmp.p, d->d);
            op->ctx->impl->sync();
        } else {
            op->impl->coef(x->d, d->d);
            op->impl->jacobi_diag_c(d->d, d->d);
        }
    });
}

// ------------------------------------------------------------------------------ multigrid
int numa_gpu_mg_create_ex(numa_gpu_ctx* ctx, size_t n, int pre, int post, int precision, int max_levels,
                          numa_gpu_mg** out) {
    if (!ctx || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto h = std::make_unique<numa_gpu_mg>();
        h->ctx = ctx;
        h->impl = std::make_unique<PoissonMG>(*ctx->impl, n, pre, post, precision, max_levels);
        *out = h.release();
    });
}

int numa_gpu_mg_create(numa_gpu_ctx* ctx, size_t n, int pre, int post, numa_gpu_mg** out) {
    return numa_gpu_mg_create_ex(ctx, n, pre, post, NUMA_GPU_FP64, 0, out);
}

int numa_gpu_mg_destroy(numa_gpu_mg* mg) {
    if (mg) {
        cudaStreamSynchronize(mg->ctx->impl->stream);
        delete mg;
    }
    return NUMA_GPU_OK;
}

int numa_gpu_mg_levels(const numa_gpu_mg* mg, size_t* levels) {
    if (!mg || !levels) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *levels = mg->impl->levels();
    return NUMA_GPU_OK;
}

int numa_gpu_mg_apply(numa_gpu_mg* mg, const numa_gpu_vec* r, numa_gpu_vec* z) {
    if (!mg) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(mg->ctx, [&] {
        same_ctx(mg->ctx, r);
        same_ctx(mg->ctx, z);
        need(r->n == mg->impl->size(), NUMA_GPU_ERR_INVALID_ARGUMENT,
             "PoissonMG received a residual of incompatible size");
        need(z->n == r->n, NUMA_GPU_ERR_SIZE_MISMATCH, "output vector length differs");
        mg->impl->apply(r->d, z->d);
    });
}

// ------------------------------------------------------------------------------ providers
int numa_gpu_provider_create_identity(numa_gpu_ctx* ctx, numa_gpu_provider** out) {
    if (!ctx || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto h = std::make_unique<numa_gpu_provider>();
        h->ctx = ctx;
        h->N = 0;
        h->impl = nullptr;
        *out = h.release();
    });
}

int numa_gpu_provider_create_poisson_mg(numa_gpu_ctx* ctx, size_t n, int pre, int post, int precision,
                                        numa_gpu_provider** out) {
    if (!ctx || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto h = std::make_unique<numa_gpu_provider>();
        h->ctx = ctx;
        h->impl = make_mg_provider(*ctx->impl, n, pre, post, precision, 0);
        h->N = n * n * n;
        *out = h.release();
    });
}

int numa_gpu_provider_create_jacobian_mg(numa_gpu_ctx* ctx, size_t n, int pre, int post, numa_gpu_provider** out) {
    if (!ctx || !out || pre < 0 || post < 1) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto h = std::make_unique<numa_gpu_provider>();
        h->ctx = ctx;
        h->impl = make_jacobian_mg_provider(*ctx->impl, n, pre, post);
        h->N = n * n * n;
        *out = h.release();
    });
}

int numa_gpu_provider_create_jacobi(numa_gpu_bratu3d* op, numa_gpu_provider** out) {
    if (!op || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(op->ctx, [&] {
        auto h = std::make_unique<numa_gpu_provider>();
        h->ctx = op->ctx;
        h->impl = make_jacobi_provider(*op->impl);
        h->N = op->impl->size();
        *out = h.release();
    });
}

int numa_gpu_provider_destroy(numa_gpu_provider* p) {
    if (p) {
        cudaStreamSynchronize(p->ctx->impl->stream);
        delete p;
    }
    return NUMA_GPU_OK;
}

int numa_gpu_provider_make(numa_gpu_provider* p, const numa_gpu_vec* x) {
    if (!p) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(p->ctx, [&] {
        same_ctx(p->ctx, x);
        if (p->N) sized(x, p->N);
        if (p->impl) p->impl->make(x->d, nullptr);
    });
}

int numa_gpu_provider_apply(numa_gpu_provider* p, const numa_gpu_vec* r, numa_gpu_vec* z) {
    if (!p) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(p->ctx, [&] {
        same_ctx(p->ctx, r);
        same_ctx(p->ctx, z);
        if (p->N) sized(r, p->N);
        need(r->n == z->n, NUMA_GPU_ERR_SIZE_MISMATCH, "output vector length differs");
        if (p->impl) p->impl->apply(r->d, z->d);
        else dev_copy(*p->ctx->impl, r->d, z->d, r->n);
    });
}

// ------------------------------------------------------------------------------ GMRES
int numa_gpu_krylov_space_create(numa_gpu_ctx* ctx, numa_gpu_krylov_space** out) {
    if (!ctx || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto h = std::make_unique<numa_gpu_krylov_space>();
        h->ctx = ctx;
        *out = h.release();
    });
}

int numa_gpu_krylov_space_destroy(numa_gpu_krylov_space* s) {
    if (s) {
        cudaStreamSynchronize(s->ctx->impl->stream);
        delete s;
    }
    return NUMA_GPU_OK;
}

int numa_gpu_krylov_space_k(const numa_gpu_krylov_space* s, size_t* k) {
    if (!s || !k) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *k = s->impl.k;
    return NUMA_GPU_OK;
}

int numa_gpu_gmres(numa_gpu_ctx* ctx, numa_gpu_apply_fn apply, void* apply_user, numa_gpu_precond_fn precond,
                   void* precond_user, const numa_gpu_vec* b, numa_gpu_vec* x, double rtol, size_t restart,
                   size_t max_iters, int zero_guess, int orth, int flexible, numa_gpu_krylov_space* save,
                   const numa_gpu_vec* r_init, numa_gmres_result* result) {
    if (!ctx || !apply || !result) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(result, 0, sizeof(*result));
    return guard(ctx, [&] {
        same_ctx(ctx, b);
        same_ctx(ctx, x);
        need(b->n == x->n, NUMA_GPU_ERR_SIZE_MISMATCH, "b and x differ in length");
        const size_t N = b->n;
        if (r_init) {
            same_ctx(ctx, r_init);
            if (r_init->n != N) {  // gmres.hpp:86-90
                result->rel_res = 1.0;
                result->breakdown = 1;
                return;
            }
        }
        if (save) need(save->ctx == ctx, NUMA_GPU_ERR_INVALID_ARGUMENT, "space belongs to another context");
        CallbackOp A;
        A.ctx = ctx;
        A.fn = apply;
        A.user = apply_user;
        A.N = N;
        CallbackPrec M;
        M.ctx = ctx;
        M.fn = precond;
        M.user = precond_user;
        M.N = N;
        GmresResult g = gmres_for(ctx, N).solve(A, precond ? &M : nullptr, b->d, x->d,
                                                gopts(rtol, restart, max_iters, zero_guess, orth, flexible),
                                                save ? &save->impl : nullptr, r_init ? r_init->d : nullptr);
        ctx->impl->sync();
        fill_gmres(g, result);
    });
}

static void bratu_jac_setup(numa_gpu_bratu3d* op, const numa_gpu_vec* xpt, int jvp_mode, BratuJacOp& J,
                            DeviceArray<double>& buf) {
    Bratu3D& f = *op->impl;
    Context& c = *op->ctx->impl;
    const size_t N = f.size();
    J.x = xpt->d;
    if (jvp_mode == NUMA_GPU_DERIV_FD) {
        buf.resize(N);
        f.eval(xpt->d, buf.p);
        dev_norm2(c, xpt->d, N, c.scalar(kSlotTmp1));
        J.fx = buf.p;
        J.xnorm = c.scalar(kSlotTmp1);
    } else if (jvp_mode == NUMA_GPU_DERIV_ANALYTIC_FP32) {
        // bound as the mixed drivers bind it: the cache of the evaluation at xpt (c, RN32(c), RN32(F))
        f.prepare_cache(NUMA_GPU_FP32);
        buf.resize(f.cache_size() + N);
        f.eval(xpt->d, buf.p + f.cache_size(), buf.p, nullptr);
        f.bind(xpt->d, buf.p, NUMA_GPU_FP32);
        J.c = buf.p;
    } else {
        need(jvp_mode == NUMA_GPU_DERIV_ANALYTIC, NUMA_GPU_ERR_INVALID_ARGUMENT, "unknown derivative mode");
        buf.resize(N);
        f.coef(xpt->d, buf.p);
        J.c = buf.p;
    }
}

int numa_gpu_gmres_bratu3d(numa_gpu_bratu3d* op, const numa_gpu_vec* xpt, int jvp_mode, numa_gpu_provider* provider,
                           const numa_gpu_vec* b, numa_gpu_vec* x, double rtol, size_t restart, size_t max_iters,
                           int zero_guess, int orth, int flexible, numa_gpu_krylov_space* save,
                           const numa_gpu_vec* r_init, numa_gmres_result* result) {
    if (!op || !result) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(result, 0, sizeof(*result));
    return guard(op->ctx, [&] {
        const size_t N = op->impl->size();
        for (const numa_gpu_vec* q : {xpt, b, (const numa_gpu_vec*)x}) {
            same_ctx(op->ctx, q);
            sized(q, N);
        }
        if (r_init) {
            same_ctx(op->ctx, r_init);
            if (r_init->n != N) {
                result->rel_res = 1.0;
                result->breakdown = 1;
                return;
            }
        }
        if (provider) {
            need(provider->ctx == op->ctx, NUMA_GPU_ERR_INVALID_ARGUMENT, "provider belongs to another context");
            need(provider->N == 0 || provider->N == N, NUMA_GPU_ERR_SIZE_MISMATCH, "provider size differs");
        }
        BratuJacOp J(*op->impl, jvp_mode);
        DeviceArray<double> buf;
        bratu_jac_setup(op, xpt, jvp_mode, J, buf);
        ProviderPrec M;
        M.p = provider ? provider->impl.get() : nullptr;
        GmresResult g = gmres_for(op->ctx, N).solve(J, M.p ? &M : nullptr, b->d, x->d,
                                                    gopts(rtol, restart, max_iters, zero_guess, orth, flexible),
                                                    save ? &save->impl : nullptr, r_init ? r_init->d : nullptr);
        op->ctx->impl->sync();
        fill_gmres(g, result);
    });
}

int numa_gpu_gmres_recycled_bratu3d(numa_gpu_bratu3d* op, const numa_gpu_vec* xpt, int jvp_mode,
                                    numa_gpu_provider* provider, const numa_gpu_vec* b, numa_gpu_vec* x, double rtol,
                                    size_t restart, size_t max_iters, int orth, const numa_gpu_krylov_space* space,
                                    numa_gpu_krylov_space* save, numa_gmres_result* result) {
    if (!op || !result || !space) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(result, 0, sizeof(*result));
    return guard(op->ctx, [&] {
        const size_t N = op->impl->size();
        for (const numa_gpu_vec* q : {xpt, b, (const numa_gpu_vec*)x}) {
            same_ctx(op->ctx, q);
            sized(q, N);
        }
        need(space->ctx == op->ctx, NUMA_GPU_ERR_INVALID_ARGUMENT, "space belongs to another context");
        BratuJacOp J(*op->impl, jvp_mode);
        DeviceArray<double> buf;
        bratu_jac_setup(op, xpt, jvp_mode, J, buf);
        ProviderPrec M;
        M.p = provider ? provider->impl.get() : nullptr;
        GmresResult g = gmres_for(op->ctx, N).solve_recycled(J, M.p ? &M : nullptr, b->d, x->d,
                                                             gopts(rtol, restart, max_iters, 1, orth, 0), space->impl,
                                                             save ? &save->impl : nullptr);
        op->ctx->impl->sync();
        fill_gmres(g, result);
    });
}

// ------------------------------------------------------------------------------ drivers
double numa_gpu_forcing(const numa_krylov_params* p, size_t k, double rnorm, double rprev, double eta_prev,
                        double res0) {
    return forcing(params_from_c(p), k, rnorm, rprev, eta_prev, res0);
}

static int run_driver(int method, numa_gpu_bratu3d* op, numa_gpu_vec* x, const numa_krylov_params* p,
                      numa_gpu_provider* provider, numa_krylov_result* result) {
    if (!op || !x || !result) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(result, 0, sizeof(*result));
    const int rc = guard(op->ctx, [&] {
        same_ctx(op->ctx, x);
        sized(x, op->impl->size());
        if (provider) {
            need(provider->ctx == op->ctx, NUMA_GPU_ERR_INVALID_ARGUMENT, "provider belongs to another context");
            need(provider->N == 0 || provider->N == x->n, NUMA_GPU_ERR_SIZE_MISMATCH, "provider size differs");
        }
        KrylovParams kp = params_from_c(p);
        Provider* pc = provider ? provider->impl.get() : nullptr;
        if (method == NUMA_GPU_METHOD_NK) newton_krylov(*op->impl, x->d, kp, pc, *result);
        else if (method == NUMA_GPU_METHOD_TF2018) tf_chebyshev_2018(*op->impl, x->d, kp, pc, *result);
        else {
            if (method == NUMA_GPU_METHOD_CHEB_REC) kp.recycle = true;
            chebyshev_inexact(*op->impl, x->d, kp, pc, *result);
        }
    });
    result->status = rc;
    return rc;
}

int numa_gpu_newton_krylov(numa_gpu_bratu3d* op, numa_gpu_vec* x, const numa_krylov_params* p,
                           numa_gpu_provider* provider, numa_krylov_result* result) {
    return run_driver(NUMA_GPU_METHOD_NK, op, x, p, provider, result);
}

int numa_gpu_chebyshev_inexact(numa_gpu_bratu3d* op, numa_gpu_vec* x, const numa_krylov_params* p,
                               numa_gpu_provider* provider, numa_krylov_result* result) {
    return run_driver(NUMA_GPU_METHOD_CHEB, op, x, p, provider, result);
}

int numa_gpu_tf_chebyshev_2018(numa_gpu_bratu3d* op, numa_gpu_vec* x, const numa_krylov_params* p,
                               numa_gpu_provider* provider, numa_krylov_result* result) {
    return run_driver(NUMA_GPU_METHOD_TF2018, op, x, p, provider, result);
}

int numa_gpu_solve_bratu3d_host(numa_gpu_ctx* ctx, size_t n, double lambda, int method, int precond_kind,
                                int mg_precision, const numa_krylov_params* p, const double* x0, double* x_out,
                                numa_krylov_result* result) {
    if (!ctx || !x0 || !x_out || !result) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(result, 0, sizeof(*result));
    const int rc = guard(ctx, [&] {
        need(n > 0 && n <= 65535, NUMA_GPU_ERR_INVALID_ARGUMENT, "grid size out of range");
        need(method >= NUMA_GPU_METHOD_NK && method <= NUMA_GPU_METHOD_TF2018, NUMA_GPU_ERR_INVALID_ARGUMENT,
             "unknown method");
        need((precond_kind >= NUMA_GPU_PRECOND_NONE && precond_kind <= NUMA_GPU_PRECOND_JACOBI) ||
                 precond_kind == NUMA_GPU_PRECOND_JACOBIAN_MG,
             NUMA_GPU_ERR_INVALID_ARGUMENT, "unknown preconditioner");
        Context& c = *ctx->impl;
        CtxExtras& e = extras(ctx);
        if (!e.host_op || e.host_n != n || e.host_lambda != lambda) {
            e.host_pc.reset();
            e.host_op = std::make_unique<Bratu3D>(c, n, lambda);
            e.host_n = n;
            e.host_lambda = lambda;
            e.host_kind = -1;
        }
        if (e.host_kind != precond_kind || e.host_prec != mg_precision || !e.host_pc) {
            if (precond_kind == NUMA_GPU_PRECOND_POISSON_MG) e.host_pc = make_mg_provider(c, n, 2, 2, mg_precision, 0);
            else if (precond_kind == NUMA_GPU_PRECOND_JACOBI) e.host_pc = make_jacobi_provider(*e.host_op);
            else if (precond_kind == NUMA_GPU_PRECOND_JACOBIAN_MG) e.host_pc = make_jacobian_mg_provider(c, n, 2, 2);
            else e.host_pc = make_identity_provider(c, n * n * n);
            e.host_kind = precond_kind;
            e.host_prec = mg_precision;
        }
        const size_t N = n * n * n;
        e.host_x.resize(N);
        // Newton–Krylov with pinned buffers overlaps the transfers with residual evaluations: x0 goes up in
        // pieces under the first one, the predicted last iterate comes down under its own
        const auto is_pinned = [](const void* ptr) {
            cudaPointerAttributes pa{};
            const bool pinned = cudaPointerGetAttributes(&pa, ptr) == cudaSuccess && pa.type == cudaMemoryTypeHost;
            cudaGetLastError();  // clears the error older runtimes report for an unregistered pointer
            return pinned;
        };
        const bool nk = method == NUMA_GPU_METHOD_NK;
        const bool pin_in = nk && is_pinned(x0), pin_out = nk && is_pinned(x_out);
        if ((pin_in || pin_out) && !e.host_up) {
            auto up = std::make_unique<HostUpload>();
            NUMA_CUDA(cudaStreamCreateWithFlags(&up->copy, cudaStreamNonBlocking));
            for (cudaEvent_t* ev : {&up->start, &up->fetch_start, &up->fetch_done})
                NUMA_CUDA(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
            for (cudaEvent_t& ev : up->done) NUMA_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            e.host_up = std::move(up);
        }
        HostUpload* up = pin_in || pin_out ? e.host_up.get() : nullptr;
        if (up) {
            up->host = pin_in ? x0 : nullptr;
            up->host_out = pin_out ? x_out : nullptr;
            up->fetched = false;
        }
        if (!pin_in) NUMA_CUDA(cudaMemcpyAsync(e.host_x.p, x0, N * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        KrylovParams kp = params_from_c(p);
        Provider* pc = e.host_pc.get();
        if (nk) newton_krylov(*e.host_op, e.host_x.p, kp, pc, *result, up);
        else if (method == NUMA_GPU_METHOD_TF2018) tf_chebyshev_2018(*e.host_op, e.host_x.p, kp, pc, *result);
        else {
            if (method == NUMA_GPU_METHOD_CHEB_REC) kp.recycle = true;
            chebyshev_inexact(*e.host_op, e.host_x.p, kp, pc, *result);
        }
        if (up && up->fetched) NUMA_CUDA(cudaEventSynchronize(up->fetch_done));
        else NUMA_CUDA(cudaMemcpyAsync(x_out, e.host_x.p, N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        c.sync();
    });
    result->status = rc;
    return rc;
}

// ------------------------------------------------------------------------------ Burgers2D
int numa_gpu_burgers2d_create(numa_gpu_ctx* ctx, size_t n, double nu, double dt, double amplitude,
                              numa_gpu_burgers2d** out) {
    if (!ctx || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto h = std::make_unique<numa_gpu_burgers2d>();
        h->ctx = ctx;
        h->impl = std::make_unique<Burgers2D>(*ctx->impl, n, nu, dt, amplitude);
        *out = h.release();
    });
}

int numa_gpu_burgers2d_destroy(numa_gpu_burgers2d* op) {
    if (op) {
        cudaStreamSynchronize(op->ctx->impl->stream);
        delete op;
    }
    return NUMA_GPU_OK;
}

int numa_gpu_burgers2d_size(const numa_gpu_burgers2d* op, size_t* N) {
    if (!op || !N) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *N = op->impl->size();
    return NUMA_GPU_OK;
}

int numa_gpu_burgers2d_cell_reynolds(const numa_gpu_burgers2d* op, double* out) {
    if (!op || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = op->impl->cell_reynolds();
    return NUMA_GPU_OK;
}

int numa_gpu_burgers2d_exact(numa_gpu_burgers2d* op, numa_gpu_vec* out) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(op->ctx, [&] {
        same_ctx(op->ctx, out);
        sized(out, op->impl->size());
        dev_copy(*op->ctx->impl, op->impl->exact(), out->d, op->impl->size());
    });
}

int numa_gpu_burgers2d_eval(numa_gpu_burgers2d* op, const numa_gpu_vec* w, numa_gpu_vec* out) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(op->ctx, [&] {
        same_ctx(op->ctx, w);
        same_ctx(op->ctx, out);
        sized(w, op->impl->size());
        sized(out, op->impl->size());
        need(w->d != out->d, NUMA_GPU_ERR_INVALID_ARGUMENT, "eval input and output must differ");
        op->impl->eval(w->d, out->d, nullptr, nullptr);
    });
}

static int burgers_derivative(numa_gpu_burgers2d* op, bool second, const numa_gpu_vec* w, const numa_gpu_vec* d,
                              numa_gpu_vec* out, int mode) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(op->ctx, [&] {
        for (const numa_gpu_vec* q : {w, d, (const numa_gpu_vec*)out}) {
            same_ctx(op->ctx, q);
            sized(q, op->impl->size());
        }
        need(out->d != w->d && out->d != d->d, NUMA_GPU_ERR_INVALID_ARGUMENT, "output must not alias an input");
        op_derivative(*op->impl, second, w->d, d->d, out->d, mode);
    });
}

int numa_gpu_burgers2d_jvp(numa_gpu_burgers2d* op, const numa_gpu_vec* w, const numa_gpu_vec* d, numa_gpu_vec* out,
                           int mode) {
    return burgers_derivative(op, false, w, d, out, mode);
}

int numa_gpu_burgers2d_d2(numa_gpu_burgers2d* op, const numa_gpu_vec* w, const numa_gpu_vec* d, numa_gpu_vec* out,
                          int mode) {
    return burgers_derivative(op, true, w, d, out, mode);
}

int numa_gpu_burgers2d_solve(numa_gpu_burgers2d* op, int method, numa_gpu_vec* x, const numa_krylov_params* p,
                             numa_gpu_provider* provider, numa_krylov_result* result) {
    if (!op || !x || !result) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(result, 0, sizeof(*result));
    const int rc = guard(op->ctx, [&] {
        check_driver_args(op->ctx, x, op->impl->size(), provider);
        dispatch_driver(method, *op->impl, x->d, p, provider ? provider->impl.get() : nullptr, *result);
    });
    result->status = rc;
    return rc;
}

// ------------------------------------------------------------------------------ HelmholtzMG2D
int numa_gpu_hmg2d_create(numa_gpu_ctx* ctx, size_t n, double alpha, double nu, int pre, int post,
                          numa_gpu_hmg2d** out) {
    if (!ctx || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto h = std::make_unique<numa_gpu_hmg2d>();
        h->ctx = ctx;
        h->impl = std::make_unique<HelmholtzMG2D>(*ctx->impl, n, alpha, nu, pre, post);
        *out = h.release();
    });
}

int numa_gpu_hmg2d_destroy(numa_gpu_hmg2d* mg) {
    if (mg) {
        cudaStreamSynchronize(mg->ctx->impl->stream);
        delete mg;
    }
    return NUMA_GPU_OK;
}

int numa_gpu_hmg2d_levels(const numa_gpu_hmg2d* mg, size_t* levels) {
    if (!mg || !levels) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *levels = mg->impl->levels();
    return NUMA_GPU_OK;
}

int numa_gpu_hmg2d_apply(numa_gpu_hmg2d* mg, const numa_gpu_vec* r, numa_gpu_vec* z) {
    if (!mg) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(mg->ctx, [&] {
        same_ctx(mg->ctx, r);
        same_ctx(mg->ctx, z);
        sized(r, mg->impl->size());
        sized(z, mg->impl->size());
        mg->impl->apply(r->d, z->d);
    });
}

int numa_gpu_provider_create_burgers_mg(numa_gpu_ctx* ctx, size_t n, double nu, double dt,
                                        numa_gpu_provider** out) {
    if (!ctx || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        need(n > 0, NUMA_GPU_ERR_INVALID_ARGUMENT, "BurgersMGProvider needs n > 0");
        need(nu > 0.0 && dt > 0.0, NUMA_GPU_ERR_INVALID_ARGUMENT, "BurgersMGProvider needs nu > 0 and dt > 0");
        auto h = std::make_unique<numa_gpu_provider>();
        h->ctx = ctx;
        h->impl = make_burgers_mg_provider(*ctx->impl, n, nu, dt, 2, 2);
        h->N = 2 * n * n;
        *out = h.release();
    });
}

int numa_gpu_solve_burgers2d_host(numa_gpu_ctx* ctx, size_t n, double nu, double dt, double amplitude, int method,
                                  int precond_kind, const numa_krylov_params* p, const double* x0, double* x_out,
                                  numa_krylov_result* result) {
    if (!ctx || !x0 || !x_out || !result) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(result, 0, sizeof(*result));
    const int rc = guard(ctx, [&] {
        need(precond_kind == NUMA_GPU_PRECOND_NONE || precond_kind == NUMA_GPU_PRECOND_BURGERS_MG,
             NUMA_GPU_ERR_INVALID_ARGUMENT, "Burgers2D takes the preconditioner NONE or BURGERS_MG");
        Context& c = *ctx->impl;
        CtxExtras& e = extras(ctx);
        if (!e.bh_op || e.bh_n != n || e.bh_nu != nu || e.bh_dt != dt || e.bh_amp != amplitude) {
            e.bh_pc.reset();
            e.bh_op = std::make_unique<Burgers2D>(c, n, nu, dt, amplitude);
            e.bh_n = n;
            e.bh_nu = nu;
            e.bh_dt = dt;
            e.bh_amp = amplitude;
            e.bh_kind = -1;
        }
        const size_t N = e.bh_op->size();
        if (e.bh_kind != precond_kind || !e.bh_pc) {
            if (precond_kind == NUMA_GPU_PRECOND_BURGERS_MG) e.bh_pc = make_burgers_mg_provider(c, n, nu, dt, 2, 2);
            else e.bh_pc = make_identity_provider(c, N);
            e.bh_kind = precond_kind;
        }
        e.bh_x.resize(N);
        NUMA_CUDA(cudaMemcpyAsync(e.bh_x.p, x0, N * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        dispatch_driver(method, *e.bh_op, e.bh_x.p, p, e.bh_pc.get(), *result);
        NUMA_CUDA(cudaMemcpyAsync(x_out, e.bh_x.p, N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        c.sync();
    });
    result->status = rc;
    return rc;
}

// ------------------------------------------------------------------------------ Brusselator1D
int numa_gpu_brusselator1d_create(numa_gpu_ctx* ctx, size_t n, double dt, numa_gpu_brusselator1d** out) {
    if (!ctx || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto h = std::make_unique<numa_gpu_brusselator1d>();
        h->ctx = ctx;
        h->impl = std::make_unique<Brusselator1D>(*ctx->impl, n, dt);
        *out = h.release();
    });
}

int numa_gpu_brusselator1d_destroy(numa_gpu_brusselator1d* op) {
    if (op) {
        cudaStreamSynchronize(op->ctx->impl->stream);
        delete op;
    }
    return NUMA_GPU_OK;
}

int numa_gpu_brusselator1d_size(const numa_gpu_brusselator1d* op, size_t* N) {
    if (!op || !N) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *N = op->impl->size();
    return NUMA_GPU_OK;
}

int numa_gpu_brusselator1d_previous(numa_gpu_brusselator1d* op, numa_gpu_vec* out) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(op->ctx, [&] {
        same_ctx(op->ctx, out);
        sized(out, op->impl->size());
        dev_copy(*op->ctx->impl, op->impl->previous(), out->d, op->impl->size());
    });
}

extern "C++" {
template <class Op>
static int op_eval(numa_gpu_ctx* ctx, Op& op, const numa_gpu_vec* w, numa_gpu_vec* out) {
    return guard(ctx, [&] {
        same_ctx(ctx, w);
        same_ctx(ctx, out);
        sized(w, op.size());
        sized(out, op.size());
        need(w->d != out->d, NUMA_GPU_ERR_INVALID_ARGUMENT, "eval input and output must differ");
        op.eval(w->d, out->d, nullptr, nullptr);
    });
}

template <class Op>
static int op_deriv(numa_gpu_ctx* ctx, Op& op, bool second, const numa_gpu_vec* w, const numa_gpu_vec* d,
                    numa_gpu_vec* out, int mode) {
    return guard(ctx, [&] {
        for (const numa_gpu_vec* q : {w, d, (const numa_gpu_vec*)out}) {
            same_ctx(ctx, q);
            sized(q, op.size());
        }
        need(out->d != w->d && out->d != d->d, NUMA_GPU_ERR_INVALID_ARGUMENT, "output must not alias an input");
        op_derivative(op, second, w->d, d->d, out->d, mode);
    });
}
}  // extern "C++"

int numa_gpu_brusselator1d_eval(numa_gpu_brusselator1d* op, const numa_gpu_vec* w, numa_gpu_vec* out) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return op_eval(op->ctx, *op->impl, w, out);
}

int numa_gpu_brusselator1d_jvp(numa_gpu_brusselator1d* op, const numa_gpu_vec* w, const numa_gpu_vec* d,
                               numa_gpu_vec* out, int mode) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return op_deriv(op->ctx, *op->impl, false, w, d, out, mode);
}

int numa_gpu_brusselator1d_d2(numa_gpu_brusselator1d* op, const numa_gpu_vec* w, const numa_gpu_vec* d,
                              numa_gpu_vec* out, int mode) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return op_deriv(op->ctx, *op->impl, true, w, d, out, mode);
}

int numa_gpu_brusselator1d_solve(numa_gpu_brusselator1d* op, int method, numa_gpu_vec* x, const numa_krylov_params* p,
                                 numa_gpu_provider* provider, numa_krylov_result* result) {
    if (!op || !x || !result) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(result, 0, sizeof(*result));
    const int rc = guard(op->ctx, [&] {
        check_driver_args(op->ctx, x, op->impl->size(), provider);
        dispatch_driver(method, *op->impl, x->d, p, provider ? provider->impl.get() : nullptr, *result);
    });
    result->status = rc;
    return rc;
}

int numa_gpu_provider_create_brusselator_jacobi(numa_gpu_brusselator1d* op, numa_gpu_provider** out) {
    if (!op || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(op->ctx, [&] {
        auto h = std::make_unique<numa_gpu_provider>();
        h->ctx = op->ctx;
        h->impl = make_bruss_jacobi_provider(*op->impl);
        h->N = op->impl->size();
        *out = h.release();
    });
}

int numa_gpu_solve_brusselator1d_host(numa_gpu_ctx* ctx, size_t n, double dt, int method, int precond_kind,
                                      const numa_krylov_params* p, const double* x0, double* x_out,
                                      numa_krylov_result* result) {
    if (!ctx || !x_out || !result) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(result, 0, sizeof(*result));
    const int rc = guard(ctx, [&] {
        need(precond_kind == NUMA_GPU_PRECOND_NONE || precond_kind == NUMA_GPU_PRECOND_BRUSS_JACOBI,
             NUMA_GPU_ERR_INVALID_ARGUMENT, "Brusselator1DStep takes the preconditioner NONE or BRUSS_JACOBI");
        Context& c = *ctx->impl;
        Brusselator1D op(c, n, dt);
        std::unique_ptr<Provider> pc = precond_kind == NUMA_GPU_PRECOND_BRUSS_JACOBI
                                           ? make_bruss_jacobi_provider(op)
                                           : make_identity_provider(c, op.size());
        const size_t N = op.size();
        DeviceArray<double> x(N);
        if (x0) NUMA_CUDA(cudaMemcpyAsync(x.p, x0, N * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        else dev_copy(c, op.previous(), x.p, N);
        dispatch_driver(method, op, x.p, p, pc.get(), *result);
        NUMA_CUDA(cudaMemcpyAsync(x_out, x.p, N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        c.sync();
    });
    result->status = rc;
    return rc;
}

// ------------------------------------------------------------------------------ Brusselator2D
int numa_gpu_brusselator2d_create(numa_gpu_ctx* ctx, size_t n, const numa_brusselator2d_params* prm,
                                  numa_gpu_brusselator2d** out) {
    if (!ctx || !out || !prm) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto h = std::make_unique<numa_gpu_brusselator2d>();
        h->ctx = ctx;
        h->impl = std::make_unique<Brusselator2D>(*ctx->impl, n, *prm);
        *out = h.release();
    });
}

int numa_gpu_brusselator2d_destroy(numa_gpu_brusselator2d* op) {
    if (op) {
        cudaStreamSynchronize(op->ctx->impl->stream);
        delete op;
    }
    return NUMA_GPU_OK;
}

int numa_gpu_brusselator2d_size(const numa_gpu_brusselator2d* op, size_t* N) {
    if (!op || !N) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *N = op->impl->size();
    return NUMA_GPU_OK;
}

int numa_gpu_brusselator2d_set_previous(numa_gpu_brusselator2d* op, const numa_gpu_vec* w) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(op->ctx, [&] {
        same_ctx(op->ctx, w);
        sized(w, op->impl->size());
        op->impl->set_previous(w->d);
    });
}

int numa_gpu_brusselator2d_eval(numa_gpu_brusselator2d* op, const numa_gpu_vec* w, numa_gpu_vec* out) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return op_eval(op->ctx, *op->impl, w, out);
}

int numa_gpu_brusselator2d_jvp(numa_gpu_brusselator2d* op, const numa_gpu_vec* w, const numa_gpu_vec* d,
                               numa_gpu_vec* out, int mode) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return op_deriv(op->ctx, *op->impl, false, w, d, out, mode);
}

int numa_gpu_brusselator2d_d2(numa_gpu_brusselator2d* op, const numa_gpu_vec* w, const numa_gpu_vec* d,
                              numa_gpu_vec* out, int mode) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return op_deriv(op->ctx, *op->impl, true, w, d, out, mode);
}

int numa_gpu_brusselator2d_solve(numa_gpu_brusselator2d* op, int method, numa_gpu_vec* x, const numa_krylov_params* p,
                                 numa_gpu_provider* provider, numa_krylov_result* result) {
    if (!op || !x || !result) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(result, 0, sizeof(*result));
    const int rc = guard(op->ctx, [&] {
        check_driver_args(op->ctx, x, op->impl->size(), provider);
        dispatch_driver(method, *op->impl, x->d, p, provider ? provider->impl.get() : nullptr, *result);
    });
    result->status = rc;
    return rc;
}

// `steps` implicit-Euler steps: each step takes the current state as the previous time level and as
// the Newton start, and leaves its solution in x.
static void advance(Brusselator2D& op, int method, size_t steps, double* x, const numa_krylov_params* p,
                    Provider* pc, numa_krylov_result* results) {
    for (size_t k = 0; k < steps; ++k) {
        op.set_previous(x);
        numa_krylov_result r;
        std::memset(&r, 0, sizeof(r));
        dispatch_driver(method, op, x, p, pc, r);
        if (results) results[k] = r;
    }
}

int numa_gpu_brusselator2d_advance(numa_gpu_brusselator2d* op, int method, size_t steps, numa_gpu_vec* x,
                                   const numa_krylov_params* p, numa_gpu_provider* provider,
                                   numa_krylov_result* results) {
    if (!op || !x) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    if (results) std::memset(results, 0, steps * sizeof(numa_krylov_result));
    return guard(op->ctx, [&] {
        check_driver_args(op->ctx, x, op->impl->size(), provider);
        advance(*op->impl, method, steps, x->d, p, provider ? provider->impl.get() : nullptr, results);
    });
}

int numa_gpu_provider_create_brusselator_mg(numa_gpu_brusselator2d* op, int precision, int pre, int post,
                                            numa_gpu_provider** out) {
    if (!op || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(op->ctx, [&] {
        auto h = std::make_unique<numa_gpu_provider>();
        h->ctx = op->ctx;
        h->impl = make_bruss_mg_provider(*op->ctx->impl, op->impl->grid(), op->impl->params(), precision, pre, post);
        h->N = op->impl->size();
        *out = h.release();
    });
}

int numa_gpu_brusselator2d_advance_host(numa_gpu_ctx* ctx, size_t n, const numa_brusselator2d_params* prm,
                                        size_t steps, int method, int precond_kind, int mg_precision,
                                        const numa_krylov_params* p, const double* x0, double* x_out,
                                        numa_krylov_result* results) {
    if (!ctx || !prm || !x0 || !x_out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    if (results) std::memset(results, 0, steps * sizeof(numa_krylov_result));
    return guard(ctx, [&] {
        need(precond_kind == NUMA_GPU_PRECOND_NONE || precond_kind == NUMA_GPU_PRECOND_BRUSS_MG,
             NUMA_GPU_ERR_INVALID_ARGUMENT, "Brusselator2D takes the preconditioner NONE or BRUSS_MG");
        Context& c = *ctx->impl;
        CtxExtras& e = extras(ctx);
        if (!e.b2_op || e.b2_n != n || std::memcmp(&e.b2_p, prm, sizeof(*prm)) != 0) {
            e.b2_pc.reset();
            e.b2_op = std::make_unique<Brusselator2D>(c, n, *prm);
            e.b2_n = n;
            e.b2_p = *prm;
            e.b2_kind = -1;
        }
        const size_t N = e.b2_op->size();
        if (e.b2_kind != precond_kind || e.b2_prec != mg_precision || !e.b2_pc) {
            if (precond_kind == NUMA_GPU_PRECOND_BRUSS_MG) e.b2_pc = make_bruss_mg_provider(c, n, *prm, mg_precision, 2, 2);
            else e.b2_pc = make_identity_provider(c, N);
            e.b2_kind = precond_kind;
            e.b2_prec = mg_precision;
        }
        e.b2_x.resize(N);
        NUMA_CUDA(cudaMemcpyAsync(e.b2_x.p, x0, N * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        advance(*e.b2_op, method, steps, e.b2_x.p, p, e.b2_pc.get(), results);
        NUMA_CUDA(cudaMemcpyAsync(x_out, e.b2_x.p, N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        c.sync();
    });
}

// ------------------------------------------------------------------------------ BrussMG2D
int numa_gpu_bmg2d_create(numa_gpu_ctx* ctx, size_t n, const numa_brusselator2d_params* prm, int precision, int pre,
                          int post, numa_gpu_bmg2d** out) {
    if (!ctx || !out || !prm) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto h = std::make_unique<numa_gpu_bmg2d>();
        h->ctx = ctx;
        h->impl = std::make_unique<BrussMG2D>(*ctx->impl, n, *prm, precision, pre, post);
        *out = h.release();
    });
}

int numa_gpu_bmg2d_destroy(numa_gpu_bmg2d* mg) {
    if (mg) {
        cudaStreamSynchronize(mg->ctx->impl->stream);
        delete mg;
    }
    return NUMA_GPU_OK;
}

int numa_gpu_bmg2d_levels(const numa_gpu_bmg2d* mg, size_t* levels) {
    if (!mg || !levels) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *levels = mg->impl->levels();
    return NUMA_GPU_OK;
}

int numa_gpu_bmg2d_set_state(numa_gpu_bmg2d* mg, const numa_gpu_vec* w) {
    if (!mg) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(mg->ctx, [&] {
        same_ctx(mg->ctx, w);
        sized(w, mg->impl->size());
        mg->impl->set_state(w->d);
    });
}

int numa_gpu_bmg2d_apply(numa_gpu_bmg2d* mg, const numa_gpu_vec* r, numa_gpu_vec* z) {
    if (!mg) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(mg->ctx, [&] {
        same_ctx(mg->ctx, r);
        same_ctx(mg->ctx, z);
        sized(r, mg->impl->size());
        sized(z, mg->impl->size());
        mg->impl->apply(r->d, z->d);
    });
}

// ------------------------------------------------------------------------------ batched solves
static std::mutex g_batch_err_mutex;
static std::string g_batch_err;

static void set_batch_error(const char* msg) {
    std::lock_guard<std::mutex> lk(g_batch_err_mutex);
    g_batch_err = msg;
}

const char* numa_gpu_batch_last_error(void) {
    std::lock_guard<std::mutex> lk(g_batch_err_mutex);
    return g_batch_err.c_str();
}

struct numa_gpu_batch {
    std::unique_ptr<BatchExecutor> impl;
};

int numa_gpu_batch_create(int device, int workers, numa_gpu_batch** out) {
    if (!out || workers < 1) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    set_batch_error("");
    try {
        auto h = std::make_unique<numa_gpu_batch>();
        h->impl = std::make_unique<BatchExecutor>(device, workers);
        *out = h.release();
        return NUMA_GPU_OK;
    } catch (const Status& s) {
        set_batch_error(s.what());
        return s.code;
    } catch (const std::exception& e) {
        set_batch_error(e.what());
        return NUMA_GPU_ERR_CUDA;
    }
}

int numa_gpu_batch_set_workers(numa_gpu_batch* b, int workers) {
    if (!b) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    try {
        b->impl->set_active(workers);
        return NUMA_GPU_OK;
    } catch (const Status& s) {
        set_batch_error(s.what());
        return s.code;
    }
}

int numa_gpu_batch_autotune(numa_gpu_batch* b, const numa_batch_instance* inst, size_t count, int method,
                            int mg_precision, const numa_krylov_params* p, const int* candidates, int ncand,
                            int* chosen, double* seconds) {
    if (!b || !inst || !count || !candidates || ncand < 1 || !chosen) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    if (method < NUMA_GPU_METHOD_NK || method > NUMA_GPU_METHOD_TF2018) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    if (mg_precision != NUMA_GPU_FP64 && mg_precision != NUMA_GPU_FP32) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < count; ++i)
        if (inst[i].n == 0 || inst[i].n > 1290) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    for (int c = 0; c < ncand; ++c)
        if (candidates[c] < 1 || candidates[c] > b->impl->workers()) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    set_batch_error("");
    try {
        *chosen = b->impl->autotune(inst, count, method, mg_precision, p, candidates, ncand, seconds);
        return NUMA_GPU_OK;
    } catch (const Status& s) {
        set_batch_error(s.what());
        return s.code;
    } catch (const std::exception& e) {
        set_batch_error(e.what());
        return NUMA_GPU_ERR_CUDA;
    }
}

int numa_gpu_batch_destroy(numa_gpu_batch* b) {
    delete b;
    return NUMA_GPU_OK;
}

int numa_gpu_batch_solve(numa_gpu_batch* b, const numa_batch_instance* inst, size_t count, int method,
                         int mg_precision, const numa_krylov_params* p, numa_batch_result* results,
                         double* wall_seconds) {
    if (!b || (count && (!inst || !results))) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    if (method < NUMA_GPU_METHOD_NK || method > NUMA_GPU_METHOD_TF2018) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    if (mg_precision != NUMA_GPU_FP64 && mg_precision != NUMA_GPU_FP32) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < count; ++i)
        if (inst[i].n == 0 || inst[i].n > 1290) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(results, 0, count * sizeof(numa_batch_result));
    set_batch_error("");
    try {
        b->impl->solve(inst, count, method, mg_precision, p, results, wall_seconds);
        return NUMA_GPU_OK;
    } catch (const Status& s) {
        set_batch_error(s.what());
        return s.code;
    } catch (const std::exception& e) {
        set_batch_error(e.what());
        return NUMA_GPU_ERR_CUDA;
    }
}

int numa_gpu_solve_batch(int device, const numa_batch_instance* inst, size_t count, int method, int mg_precision,
                         const numa_krylov_params* p, int workers, numa_batch_result* results,
                         double* wall_seconds) {
    if ((count && (!inst || !results)) || workers < 1) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    if (method < NUMA_GPU_METHOD_NK || method > NUMA_GPU_METHOD_TF2018) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    if (mg_precision != NUMA_GPU_FP64 && mg_precision != NUMA_GPU_FP32) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < count; ++i)
        if (inst[i].n == 0 || inst[i].n > 1290) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(results, 0, count * sizeof(numa_batch_result));
    set_batch_error("");
    try {
        BatchExecutor ex(device, workers);
        ex.solve(inst, count, method, mg_precision, p, results, wall_seconds);
        return NUMA_GPU_OK;
    } catch (const Status& s) {
        set_batch_error(s.what());
        return s.code;
    } catch (const std::bad_alloc&) {
        set_batch_error("host allocation failed");
        return NUMA_GPU_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        set_batch_error(e.what());
        return NUMA_GPU_ERR_CUDA;
    }
}

// ------------------------------------------------------------------------------ diagnostics
int numa_gpu_diag_fp64_peak(numa_gpu_ctx* ctx, double* tflops) {
    if (!ctx || !tflops) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(ctx, [&] { *tflops = diag_fp64_peak_tflops(*ctx->impl); });
}

int numa_gpu_diag_exp(const numa_gpu_vec* x, numa_gpu_vec* out, numa_gpu_vec* cuda_ref) {
    if (!x || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(x->ctx, [&] {
        same_ctx(x->ctx, out);
        need(out->n == x->n, NUMA_GPU_ERR_SIZE_MISMATCH, "output length differs");
        need(out->d != x->d, NUMA_GPU_ERR_INVALID_ARGUMENT, "output must not alias the input");
        if (cuda_ref) {
            same_ctx(x->ctx, cuda_ref);
            need(cuda_ref->n == x->n, NUMA_GPU_ERR_SIZE_MISMATCH, "reference length differs");
        }
        diag_exp(*x->ctx->impl, x->d, out->d, cuda_ref ? cuda_ref->d : nullptr, x->n);
    });
}

int numa_gpu_diag_div(const numa_gpu_vec* a, double b, numa_gpu_vec* out) {
    if (!a || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(a->ctx, [&] {
        same_ctx(a->ctx, out);
        need(out->n == a->n, NUMA_GPU_ERR_SIZE_MISMATCH, "output length differs");
        diag_div(*a->ctx->impl, a->d, b, out->d, a->n);
    });
}

int numa_gpu_diag_conv3d_wgrad(numa_gpu_ctx* ctx, size_t n, int cin, int cout, const float* x, const float* g,
                               float* dw, float* db) {
    if (!ctx || !x || !g || !dw || !db || n == 0 || n > 63) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(ctx, [&] { diag_conv3d_wgrad(*ctx->impl, (int)n, cin, cout, x, g, dw, db); });
}

int numa_gpu_diag_conv3d(numa_gpu_ctx* ctx, size_t n, int cin, int cout, int adjoint, const float* x,
                         const float* w, const float* bias, float* y) {
    if (!ctx || !x || !w || !y) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(ctx, [&] {
        need(n >= 1 && n <= 63, NUMA_GPU_ERR_INVALID_ARGUMENT, "grid size must be in 1..63");
        diag_conv3d(*ctx->impl, (int)n, cin, cout, adjoint, x, w, bias, y);
    });
}

// ------------------------------------------------------------------------------ learned preconditioner
int numa_gpu_learned_create(numa_gpu_ctx* ctx, size_t n0, uint64_t seed, numa_gpu_learned** out) {
    if (!ctx || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto h = std::make_unique<numa_gpu_learned>();
        h->ctx = ctx;
        h->impl = learned_create(*ctx->impl, (int)n0, seed);
        *out = h.release();
    });
}

int numa_gpu_learned_destroy(numa_gpu_learned* net) {
    if (net) {
        cudaStreamSynchronize(net->ctx->impl->stream);
        delete net;
    }
    return NUMA_GPU_OK;
}

int numa_gpu_learned_num_params(const numa_gpu_learned* net, size_t* n) {
    if (!net || !n) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *n = learned_num_params(*net->impl);
    return NUMA_GPU_OK;
}

int numa_gpu_learned_get_params(numa_gpu_learned* net, float* host, size_t n) {
    if (!net || !host) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(net->ctx, [&] {
        need(n == learned_num_params(*net->impl), NUMA_GPU_ERR_SIZE_MISMATCH, "parameter count differs");
        learned_get_params(*net->impl, host);
    });
}

int numa_gpu_learned_set_params(numa_gpu_learned* net, const float* host, size_t n) {
    if (!net || !host) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(net->ctx, [&] {
        need(n == learned_num_params(*net->impl), NUMA_GPU_ERR_SIZE_MISMATCH, "parameter count differs");
        learned_set_params(*net->impl, host);
    });
}

int numa_gpu_learned_forward(numa_gpu_learned* net, const float* features, float* out) {
    if (!net || !features || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(net->ctx, [&] { learned_forward_host(*net->ctx->impl, *net->impl, features, out); });
}

int numa_gpu_learned_gradient(numa_gpu_learned* net, const float* features, const float* target, float* loss,
                              float* grad) {
    if (!net || !features || !target || !loss || !grad) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(net->ctx, [&] { learned_grad_host(*net->ctx->impl, *net->impl, features, target, loss, grad); });
}

int numa_gpu_learned_train(numa_gpu_learned* net, const numa_learned_train_params* p,
                           numa_learned_train_report* report) {
    if (!net || !p || !report) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(report, 0, sizeof(*report));
    return guard(net->ctx, [&] {
        need(p->instances > 0 && p->states > 0 && p->rhs_per_state >= 0 && p->epochs >= 0 && p->batch > 0,
             NUMA_GPU_ERR_INVALID_ARGUMENT, "invalid training sizes");
        need(p->lambda_max >= p->lambda_min && p->solve_rtol > 0.0 && p->lr > 0.0f, NUMA_GPU_ERR_INVALID_ARGUMENT,
             "invalid training parameters");
        learned_train(*net->ctx->impl, *net->impl, *p, *report);
    });
}

int numa_gpu_provider_create_learned(numa_gpu_ctx* ctx, size_t n, numa_gpu_learned* net, double stall,
                                     numa_gpu_provider** out) {
    if (!ctx || !net || !out) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        need(net->ctx == ctx, NUMA_GPU_ERR_INVALID_ARGUMENT, "network belongs to another context");
        need(stall > 0.0, NUMA_GPU_ERR_INVALID_ARGUMENT, "stall factor must be positive");
        auto h = std::make_unique<numa_gpu_provider>();
        h->ctx = ctx;
        h->impl = make_learned_provider(*ctx->impl, n, *net->impl, stall);
        h->N = n * n * n;
        *out = h.release();
    });
}

int numa_gpu_provider_learned_stats(numa_gpu_provider* p, size_t* applies, size_t* fallbacks) {
    if (!p || !applies || !fallbacks) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(p->ctx, [&] {
        need(p->impl != nullptr, NUMA_GPU_ERR_INVALID_ARGUMENT, "not a learned preconditioner");
        learned_provider_stats(*p->impl, applies, fallbacks);
    });
}

int numa_gpu_diag_time_bmg2d_pass(numa_gpu_bmg2d* mg, int reps, double* ms_per_pass) {
    if (!mg || !ms_per_pass || reps < 1) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(mg->ctx, [&] { *ms_per_pass = mg->impl->time_finest_pass(reps); });
}

struct numa_gpu_bsolver {
    numa_gpu_ctx* ctx;
    std::unique_ptr<BatchSolver> impl;
};

int numa_gpu_bsolver_create(numa_gpu_ctx* ctx, const numa_batch_instance* inst, size_t count,
                            const numa_krylov_params* p, numa_gpu_bsolver** out) {
    if (!ctx || !out || !inst || count == 0) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        auto h = std::make_unique<numa_gpu_bsolver>();
        h->ctx = ctx;
        h->impl = std::make_unique<BatchSolver>(*ctx->impl, inst, count, params_from_c(p));
        *out = h.release();
    });
}

int numa_gpu_bsolver_destroy(numa_gpu_bsolver* s) {
    if (!s) return NUMA_GPU_OK;
    numa_gpu_ctx* ctx = s->ctx;
    return guard(ctx, [&] { delete s; });
}

int numa_gpu_bsolver_solve(numa_gpu_bsolver* s, double* x_out, numa_batch_result* results, double* seconds) {
    if (!s || !results) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(s->ctx, [&] { s->impl->solve(x_out, results, seconds); });
}

int numa_gpu_bsolver_get_tuning(const numa_gpu_bsolver* s, numa_batch_tuning* t) {
    if (!s || !t) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    std::memset(t, 0, sizeof(*t));
    const BatchTuning b = s->impl->tuning();
    t->planes = b.planes;
    t->elems_per_block = b.elems_per_block;
    return NUMA_GPU_OK;
}

int numa_gpu_bsolver_set_tuning(numa_gpu_bsolver* s, const numa_batch_tuning* t) {
    if (!s || !t || t->planes < 1 || t->elems_per_block < 1) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(s->ctx, [&] { s->impl->set_tuning(BatchTuning{t->planes, t->elems_per_block}); });
}

int numa_gpu_bsolver_autotune(numa_gpu_bsolver* s, const int* planes, int np, const int* elems, int ne,
                              numa_batch_tuning* chosen, double* seconds) {
    if (!s || !planes || !elems || np < 1 || ne < 1) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    for (int a = 0; a < np; ++a)
        if (planes[a] < 1) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    for (int b = 0; b < ne; ++b)
        if (elems[b] < 1) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(s->ctx, [&] {
        const BatchTuning b = s->impl->autotune(planes, np, elems, ne, seconds);
        if (chosen) {
            std::memset(chosen, 0, sizeof(*chosen));
            chosen->planes = b.planes;
            chosen->elems_per_block = b.elems_per_block;
        }
    });
}

int numa_gpu_diag_time_smoother(numa_gpu_mg* mg, int reps, double* ms_per_pass) {
    if (!mg || !ms_per_pass || reps < 1) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(mg->ctx, [&] { *ms_per_pass = mg->impl->time_finest_pass(reps); });
}

int numa_gpu_diag_eval(numa_gpu_bratu3d* op, const numa_gpu_vec* x, int precision, numa_gpu_vec* out, double* norm) {
    if (!op) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    if (precision != NUMA_GPU_FP64 && precision != NUMA_GPU_FP32) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(op->ctx, [&] {
        same_ctx(op->ctx, x);
        same_ctx(op->ctx, out);
        sized(x, op->impl->size());
        sized(out, op->impl->size());
        need(out->d != x->d, NUMA_GPU_ERR_INVALID_ARGUMENT, "eval output must not alias its input");
        op->impl->eval_as(x->d, precision, out->d, norm);
    });
}

int numa_gpu_diag_time_eval(numa_gpu_bratu3d* op, const numa_gpu_vec* x, int precision, int reps, double* ms_per_eval) {
    if (!op || !ms_per_eval || reps < 1) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    if (precision != NUMA_GPU_FP64 && precision != NUMA_GPU_FP32) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    return guard(op->ctx, [&] {
        same_ctx(op->ctx, x);
        sized(x, op->impl->size());
        *ms_per_eval = op->impl->time_eval(x->d, precision, reps);
    });
}

}  // extern "C"
