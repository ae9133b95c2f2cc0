/*
 * numa_gpu.h — C ABI of libnuma_gpu.so, the GB300 (sm_103a) implementation of the
 * matrix-free nonlinear-solve path of kapumota/chebyshev-nonlinear-lab (namespace numa::op).
 *
 * The reference exposes this path as header-only C++20 templates with no ABI.  Each entry
 * point below replaces one of those interfaces; the citation beside it names the reference
 * file:line whose behaviour it reproduces (paths relative to the reference project root).
 *
 * Conventions (shared by every function):
 *   - Every function returns an int status: NUMA_GPU_OK (0) or a numa_gpu_status code.
 *     Numerical failure is NOT an error status: it is reported in the result structs
 *     (converged / breakdown / n_lin_failures), exactly as the reference does.
 *   - Handles own device memory; *_destroy frees it.  Host buffers belong to the caller.
 *   - All work is stream-ordered on the context's stream; calls that return a scalar or a
 *     result struct to the host synchronise that stream first.
 *   - Objects are not thread-safe (the reference's PoissonMG keeps mutable work arrays,
 *     linalg/poisson_mg.hpp:11); one host thread drives one context.
 *   - Vectors are FP64, lexicographic (i*n + j)*n + k with k fastest (problems/bratu3d.hpp:85),
 *     Dirichlet boundary values implicit (no ghost layer).
 */
#ifndef NUMA_GPU_H
#define NUMA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NUMA_GPU_ABI_VERSION 1

/* ---------------------------------------------------------------- status codes */
typedef enum numa_gpu_status {
    NUMA_GPU_OK = 0,
    NUMA_GPU_ERR_INVALID_ARGUMENT = 1, /* std::invalid_argument in PoissonMG (poisson_mg.hpp:29-36, :71-74) */
    NUMA_GPU_ERR_OVERFLOW = 2,         /* std::overflow_error in PoissonMG (poisson_mg.hpp:38-42) */
    NUMA_GPU_ERR_SIZE_MISMATCH = 3,    /* vector lengths disagree with the operator size */
    NUMA_GPU_ERR_CUDA = 4,             /* a CUDA runtime call failed; see numa_gpu_last_error */
    NUMA_GPU_ERR_OUT_OF_MEMORY = 5,
    NUMA_GPU_ERR_NO_DEVICE = 6,
    NUMA_GPU_ERR_CALLBACK = 7,         /* a user apply/precond callback returned non-zero */
    NUMA_GPU_ERR_NOT_SUPPORTED = 8,
    NUMA_GPU_ERR_TOO_LARGE = 9         /* the problem does not fit a fixed-size scratch array */
} numa_gpu_status;

/* ---------------------------------------------------------------- enums */
typedef enum numa_gpu_precision {
    NUMA_GPU_FP64 = 0,
    NUMA_GPU_FP32 = 1
} numa_gpu_precision;

/* How a directional derivative is formed. */
typedef enum numa_gpu_deriv_mode {
    NUMA_GPU_DERIV_ANALYTIC = 0,     /* Bratu3D::jvp / Bratu3D::d2 (problems/bratu3d.hpp:33-56) */
    NUMA_GPU_DERIV_FD = 1,           /* jvp_fd / d2_fd (operators/operator.hpp:100-134) */
    NUMA_GPU_DERIV_ANALYTIC_FP32 = 2, /* extension, jvp only: the analytic product in FP32 arithmetic
                                        (Bratu3D, Brusselator2D; FP64 for operators without one) */
    NUMA_GPU_DERIV_ANALYTIC_FP32X = 3 /* extension, Bratu3D jvp only: the analytic product of RN32(v) to
                                        FP64 accuracy (double-FP32 stencil, FP64 lambda e^x), as the
                                        mixed path's tight linear solves take it (jvp_tight) */
} numa_gpu_deriv_mode;

/* Arnoldi orthogonalisation. */
typedef enum numa_gpu_orth {
    NUMA_GPU_ORTH_MGS = 0, /* modified Gram-Schmidt, the reference (linalg/gmres.hpp:141-144) */
    NUMA_GPU_ORTH_CGS2 = 1, /* classical Gram-Schmidt with one reorthogonalisation, fused multi-dot */
    NUMA_GPU_ORTH_CGS1 = 2  /* classical Gram-Schmidt, one pass (multi-dot, then update and norm) */
} numa_gpu_orth;

/* Nonlinear methods of the reference's R1 drivers. */
typedef enum numa_gpu_method {
    NUMA_GPU_METHOD_NK = 0,       /* newton_krylov (methods/krylov_newton.hpp:69-114) */
    NUMA_GPU_METHOD_CHEB = 1,     /* chebyshev_inexact (krylov_newton.hpp:116-189) */
    NUMA_GPU_METHOD_CHEB_REC = 2, /* chebyshev_inexact with recycle = true */
    NUMA_GPU_METHOD_TF2018 = 3    /* tf_chebyshev_2018 (methods/tf_chebyshev_2018.hpp:52-132) */
} numa_gpu_method;

/* Preconditioner providers (the reference's Provider::make(x) -> Bound protocol). */
typedef enum numa_gpu_precond_kind {
    NUMA_GPU_PRECOND_NONE = 0,       /* NoPrecond / IdentityPrecond (krylov_newton.hpp:20-22, gmres.hpp:37-39) */
    NUMA_GPU_PRECOND_POISSON_MG = 1, /* PoissonMGProvider (linalg/poisson_mg.hpp:303-320) */
    NUMA_GPU_PRECOND_JACOBI = 2,     /* BratuJacobi (problems/bratu3d.hpp:104-120) */
    NUMA_GPU_PRECOND_BURGERS_MG = 3, /* BurgersMGProvider (problems/burgers2d.hpp:220-246) */
    NUMA_GPU_PRECOND_LEARNED = 4,    /* extension: FP32 V-cycle + learned coarse correction (FGMRES) */
    NUMA_GPU_PRECOND_BRUSS_JACOBI = 5, /* BrusselatorJacobi (problems/brusselator1d.hpp:194-222) */
    NUMA_GPU_PRECOND_BRUSS_MG = 6,     /* extension: periodic coupled-block multigrid of Brusselator2D */
    NUMA_GPU_PRECOND_JACOBIAN_MG = 7   /* extension: FP32 V-cycle with Jacobian-aware coarse levels */
} numa_gpu_precond_kind;

/* ---------------------------------------------------------------- parameter / result structs */

/* Parameters of the periodic 2D Brusselator step (reaction terms of problems/brusselator1d.hpp:4-10). */
typedef struct numa_brusselator2d_params {
    double A, B;   /* reaction constants                               (1, 3.4) */
    double Du, Dv; /* diffusion coefficients of u and v                (0.002, 0.002) */
    double dt;     /* implicit-Euler step                              (0.01) */
} numa_brusselator2d_params;

/* KrylovParams (methods/krylov_newton.hpp:24-38), field for field, plus GPU extensions whose
 * zero value is the reference behaviour. */
typedef struct numa_krylov_params {
    double rtol_nl;            /* ||F|| <= rtol_nl * ||F(x0)||            default 1e-8 */
    uint64_t max_nl;           /*                                           default 50 */
    double eta_init;           /*                                           default 0.5 */
    double eta_max;            /*                                           default 0.9 */
    double gamma;              /* Eisenstat-Walker choice 2                 default 0.9 */
    double alpha;              /*                                           default 2.0 */
    double eta2_factor;        /* tolerance of the second Chebyshev solve   default 10 */
    double eta2_max;           /*                                           default 0.5 */
    uint64_t gmres_restart;    /*                                           default 50 */
    uint64_t gmres_max_iters;  /*                                           default 500 */
    double armijo;             /*                                           default 1e-4 */
    double min_lambda;         /*                                           default 1e-4 */
    int32_t recycle;           /* recycle the Krylov space between the two Chebyshev solves */
    /* --- extensions (0 = reference behaviour) --- */
    int32_t jvp_mode;          /* numa_gpu_deriv_mode of the Krylov matvec */
    int32_t d2_mode;           /* numa_gpu_deriv_mode of F''(x)[z,z] */
    int32_t orth;              /* numa_gpu_orth */
    int32_t flexible;          /* 1 = FGMRES (stores Z_j = M^-1 v_j; no extra precond per cycle) */
    int32_t jvp_precision;     /* numa_gpu_precision of the Krylov matvec arithmetic */
    int32_t jvp_tight;         /* 1 = with jvp_precision FP32, linear solves whose tolerance is below 1e-5
                                  take the product of each FP32 preconditioned vector to FP64 accuracy
                                  (double-FP32 stencil, FP64 coefficient) where the operator offers it
                                  (Bratu3D): rounded once to FP32 into the FP32 Arnoldi basis down to a
                                  tolerance of 1e-6, with an FP64 basis below; 0 = FP32 arithmetic */
    int32_t coarse_jacobian;   /* batched solver only (numa_gpu_bsolver_*): 1 = its FP32 multigrid's levels
                                  n <= 15 solve with the Jacobian -Lap_h - lambda e^u of each iterate, as
                                  numa_gpu_provider_create_jacobian_mg does for one instance; 0 = Poisson */
    int32_t reserved[2];
} numa_krylov_params;

/* KrylovResult (krylov_newton.hpp:40-49) without x (the solution is written into the caller's
 * vector), plus the per-primitive timers of operators/timing.hpp:16-24 (seconds; measured with
 * CUDA events on the context stream when timing is enabled, else 0). */
typedef struct numa_krylov_result {
    int32_t converged;
    int32_t status;            /* NUMA_GPU_OK, or the error that ended the solve */
    uint64_t iters;
    uint64_t n_F;
    uint64_t n_JVP;
    uint64_t n_D2;
    uint64_t n_lin_iters;
    uint64_t n_lin_failures;
    uint64_t n_prec;
    double res0;
    double res;
    double t_F;
    double t_JVP;
    double t_D2;
    double t_prec;
    double t_setup_dynamic;
    double t_total;
} numa_krylov_result;

/* GmresResult (linalg/gmres.hpp:14-21). */
typedef struct numa_gmres_result {
    uint64_t iters;
    uint64_t matvecs;
    uint64_t precs;
    double rel_res;
    int32_t converged;
    int32_t breakdown;
} numa_gmres_result;

/* ---------------------------------------------------------------- opaque handles */
typedef struct numa_gpu_ctx numa_gpu_ctx;
typedef struct numa_gpu_vec numa_gpu_vec;
typedef struct numa_gpu_bratu3d numa_gpu_bratu3d;
typedef struct numa_gpu_mg numa_gpu_mg;
typedef struct numa_gpu_provider numa_gpu_provider;
typedef struct numa_gpu_krylov_space numa_gpu_krylov_space;
typedef struct numa_gpu_burgers2d numa_gpu_burgers2d;
typedef struct numa_gpu_hmg2d numa_gpu_hmg2d;
typedef struct numa_gpu_brusselator1d numa_gpu_brusselator1d;
typedef struct numa_gpu_brusselator2d numa_gpu_brusselator2d;
typedef struct numa_gpu_bmg2d numa_gpu_bmg2d;
typedef struct numa_gpu_learned numa_gpu_learned;

/* ---------------------------------------------------------------- library / context */
int numa_gpu_abi_version(void);
const char* numa_gpu_status_string(int status);
void numa_krylov_params_default(numa_krylov_params* p);  /* KrylovParams{} defaults */

int numa_gpu_ctx_create(int device, numa_gpu_ctx** out);
/* Destroy every object created on a context (vectors, operators, hierarchies, providers, Krylov
 * spaces, solvers) before the context: their destroy functions use the context's stream. */
int numa_gpu_ctx_destroy(numa_gpu_ctx* ctx);
int numa_gpu_ctx_synchronize(numa_gpu_ctx* ctx);
/* Message of the last failing call on this context ("" if none). */
const char* numa_gpu_ctx_last_error(numa_gpu_ctx* ctx);
/* 1 = record per-primitive CUDA-event timers into numa_krylov_result (adds event records). */
int numa_gpu_ctx_set_timing(numa_gpu_ctx* ctx, int enable);
/* Number of kernels this library launched on the context since creation / the last reset. */
int numa_gpu_ctx_kernel_launches(numa_gpu_ctx* ctx, uint64_t* out);
int numa_gpu_ctx_reset_kernel_launches(numa_gpu_ctx* ctx);
/* The context's cudaStream_t, as an opaque pointer (for callers that order their own work). */
int numa_gpu_ctx_stream(numa_gpu_ctx* ctx, void** stream_out);

/* ---------------------------------------------------------------- device vectors (DVec) */
int numa_gpu_vec_create(numa_gpu_ctx* ctx, size_t n, numa_gpu_vec** out);
int numa_gpu_vec_destroy(numa_gpu_vec* v);
int numa_gpu_vec_size(const numa_gpu_vec* v, size_t* n);
int numa_gpu_vec_device_ptr(numa_gpu_vec* v, double** dptr);
int numa_gpu_vec_upload(numa_gpu_vec* v, const double* host, size_t n);
int numa_gpu_vec_download(const numa_gpu_vec* v, double* host, size_t n);
int numa_gpu_vec_fill(numa_gpu_vec* v, double value);
int numa_gpu_vec_copy(const numa_gpu_vec* src, numa_gpu_vec* dst);
/* BLAS-1 of operators/operator.hpp:19-41. */
int numa_gpu_vec_dot(const numa_gpu_vec* a, const numa_gpu_vec* b, double* out);   /* dot   :19-27 */
int numa_gpu_vec_norm2(const numa_gpu_vec* a, double* out);                        /* norm2 :29 */
int numa_gpu_vec_axpy(double a, const numa_gpu_vec* x, numa_gpu_vec* y);           /* axpy  :32-41 */

/* ---------------------------------------------------------------- Bratu3D operator */
/* Bratu3D(n, lambda) (problems/bratu3d.hpp:12-16). */
int numa_gpu_bratu3d_create(numa_gpu_ctx* ctx, size_t n, double lambda, numa_gpu_bratu3d** out);
int numa_gpu_bratu3d_destroy(numa_gpu_bratu3d* op);
int numa_gpu_bratu3d_size(const numa_gpu_bratu3d* op, size_t* N);
/* out = F(x)                          Bratu3D::eval (bratu3d.hpp:21-31) */
int numa_gpu_bratu3d_eval(numa_gpu_bratu3d* op, const numa_gpu_vec* x, numa_gpu_vec* out);
/* out = F'(x) v   mode ANALYTIC: Bratu3D::jvp (bratu3d.hpp:33-43); FD: jvp_fd (operator.hpp:101-114) */
int numa_gpu_bratu3d_jvp(numa_gpu_bratu3d* op, const numa_gpu_vec* x, const numa_gpu_vec* v,
                         numa_gpu_vec* out, int mode);
/* out = F''(x)[v,v] mode ANALYTIC: Bratu3D::d2 (bratu3d.hpp:46-56); FD: d2_fd (operator.hpp:118-134) */
int numa_gpu_bratu3d_d2(numa_gpu_bratu3d* op, const numa_gpu_vec* x, const numa_gpu_vec* v,
                        numa_gpu_vec* out, int mode);
/* d = 6 h^-2 - lambda e^x             Bratu3D::jacobi_diag (bratu3d.hpp:59-69) */
int numa_gpu_bratu3d_jacobi_diag(numa_gpu_bratu3d* op, const numa_gpu_vec* x, numa_gpu_vec* d);

/* ---------------------------------------------------------------- Burgers2D operator */
/* Burgers2D(n, nu, dt, amplitude) (problems/burgers2d.hpp:23-52): one implicit-Euler step of 2D
 * viscous Burgers with the manufactured root w*; N = 2 n^2, w = (u, v) component-major. */
int numa_gpu_burgers2d_create(numa_gpu_ctx* ctx, size_t n, double nu, double dt, double amplitude,
                              numa_gpu_burgers2d** out);
int numa_gpu_burgers2d_destroy(numa_gpu_burgers2d* op);
int numa_gpu_burgers2d_size(const numa_gpu_burgers2d* op, size_t* N);
/* |amplitude| / (nu (n + 1))           Burgers2D::cell_reynolds (burgers2d.hpp:59-62) */
int numa_gpu_burgers2d_cell_reynolds(const numa_gpu_burgers2d* op, double* out);
/* out = w*                             Burgers2D::exact (burgers2d.hpp:63) */
int numa_gpu_burgers2d_exact(numa_gpu_burgers2d* op, numa_gpu_vec* out);
/* out = F(w)                           Burgers2D::eval (burgers2d.hpp:65-69) */
int numa_gpu_burgers2d_eval(numa_gpu_burgers2d* op, const numa_gpu_vec* w, numa_gpu_vec* out);
/* out = F'(w) d   mode ANALYTIC: Burgers2D::jvp (burgers2d.hpp:71-123); FD: jvp_fd */
int numa_gpu_burgers2d_jvp(numa_gpu_burgers2d* op, const numa_gpu_vec* w, const numa_gpu_vec* d,
                           numa_gpu_vec* out, int mode);
/* out = F''(w)[d,d] mode ANALYTIC: Burgers2D::d2 (burgers2d.hpp:125-160); FD: d2_fd */
int numa_gpu_burgers2d_d2(numa_gpu_burgers2d* op, const numa_gpu_vec* w, const numa_gpu_vec* d,
                          numa_gpu_vec* out, int mode);

/* ---------------------------------------------------------------- Poisson multigrid */
/* PoissonMG(n, pre, post) (linalg/poisson_mg.hpp:26-64): levels while n is odd, down to 1. */
int numa_gpu_mg_create(numa_gpu_ctx* ctx, size_t n, int pre, int post, numa_gpu_mg** out);
/* Extension: precision of the V-cycle arithmetic (FP64 = reference) and a cap on the level
 * count (0 = the reference hierarchy). */
int numa_gpu_mg_create_ex(numa_gpu_ctx* ctx, size_t n, int pre, int post, int precision,
                          int max_levels, numa_gpu_mg** out);
int numa_gpu_mg_destroy(numa_gpu_mg* mg);
int numa_gpu_mg_levels(const numa_gpu_mg* mg, size_t* levels);    /* PoissonMG::levels :66 */
/* z = one V-cycle applied to r        PoissonMG::operator() (poisson_mg.hpp:69-80) */
int numa_gpu_mg_apply(numa_gpu_mg* mg, const numa_gpu_vec* r, numa_gpu_vec* z);

/* ---------------------------------------------------------------- 2D Helmholtz multigrid */
/* HelmholtzMG2D(n, alpha, nu, pre, post) (linalg/helmholtz_mg2d.hpp:13-32): V-cycle for
 * alpha I - nu Lap_h on n^2 points, levels while n is odd; FP64, bit-identical to the reference. */
int numa_gpu_hmg2d_create(numa_gpu_ctx* ctx, size_t n, double alpha, double nu, int pre, int post,
                          numa_gpu_hmg2d** out);
int numa_gpu_hmg2d_destroy(numa_gpu_hmg2d* mg);
int numa_gpu_hmg2d_levels(const numa_gpu_hmg2d* mg, size_t* levels);  /* levels() :34 */
/* z = one V-cycle applied to r          HelmholtzMG2D::operator() (helmholtz_mg2d.hpp:36-42) */
int numa_gpu_hmg2d_apply(numa_gpu_hmg2d* mg, const numa_gpu_vec* r, numa_gpu_vec* z);

/* ---------------------------------------------------------------- preconditioner providers */
/* Provider::make(x) -> Bound, Bound(r, z) (krylov_newton.hpp:20-22, poisson_mg.hpp:303-320,
 * bratu3d.hpp:104-120).  A provider owns what it creates (the MG hierarchy, the diagonal). */
int numa_gpu_provider_create_identity(numa_gpu_ctx* ctx, numa_gpu_provider** out);
int numa_gpu_provider_create_poisson_mg(numa_gpu_ctx* ctx, size_t n, int pre, int post, int precision,
                                        numa_gpu_provider** out);
int numa_gpu_provider_create_jacobi(numa_gpu_bratu3d* op, numa_gpu_provider** out);
/* No counterpart in the reference (whose PoissonMGProvider, linalg/poisson_mg.hpp:303-320, ignores
 * the iterate): the FP32 PoissonMG V-cycle whose coarse levels n <= 15 (the one-CTA tail) solve with
 * the Jacobian -Lap_h - c instead of -Lap_h, c the full-weighting restriction of the Bratu3D
 * coefficient lambda e^u of the iterate the provider is bound at (make reads the operator's cache).
 * The fine levels keep the Poisson smoother: the shift matters only for the smooth modes, which the
 * coarse levels carry.  n = 2^k - 1 >= 31 (an odd hierarchy down to the tail). */
int numa_gpu_provider_create_jacobian_mg(numa_gpu_ctx* ctx, size_t n, int pre, int post, numa_gpu_provider** out);
/* BurgersMGProvider(n, nu, dt): HelmholtzMG2D(n, 1/dt, nu) V(2,2) on u and on v. */
int numa_gpu_provider_create_burgers_mg(numa_gpu_ctx* ctx, size_t n, double nu, double dt,
                                        numa_gpu_provider** out);
int numa_gpu_provider_destroy(numa_gpu_provider* p);
int numa_gpu_provider_make(numa_gpu_provider* p, const numa_gpu_vec* x);            /* make(x)  */
int numa_gpu_provider_apply(numa_gpu_provider* p, const numa_gpu_vec* r, numa_gpu_vec* z); /* Bound(r,z) */

/* ---------------------------------------------------------------- GMRES */
/* KrylovSpace (gmres.hpp:25-35): Arnoldi basis of the last cycle, kept on the device. */
int numa_gpu_krylov_space_create(numa_gpu_ctx* ctx, numa_gpu_krylov_space** out);
int numa_gpu_krylov_space_destroy(numa_gpu_krylov_space* s);
int numa_gpu_krylov_space_k(const numa_gpu_krylov_space* s, size_t* k);

/* User callbacks on device vectors: apply computes out = A v, precond computes z = M^-1 r.
 * Return 0 on success. */
typedef int (*numa_gpu_apply_fn)(void* user, const numa_gpu_vec* v, numa_gpu_vec* out);
typedef int (*numa_gpu_precond_fn)(void* user, const numa_gpu_vec* r, numa_gpu_vec* z);

/* gmres(apply, precond, b, x, rtol, restart, max_iters, zero_guess, save, r_init)
 * (linalg/gmres.hpp:61-223).  precond may be NULL (IdentityPrecond).  save and r_init may be
 * NULL.  orth selects MGS (reference) or CGS2; flexible = 1 selects FGMRES. */
int numa_gpu_gmres(numa_gpu_ctx* ctx, numa_gpu_apply_fn apply, void* apply_user,
                   numa_gpu_precond_fn precond, void* precond_user,
                   const numa_gpu_vec* b, numa_gpu_vec* x, double rtol, size_t restart,
                   size_t max_iters, int zero_guess, int orth, int flexible,
                   numa_gpu_krylov_space* save, const numa_gpu_vec* r_init,
                   numa_gmres_result* result);
/* The same with the Bratu3D Jacobian at xpt as A (apply = f.jvp(xpt, .), mode = jvp mode) and a
 * bound provider as M (provider may be NULL): the form the nonlinear drivers use internally. */
int numa_gpu_gmres_bratu3d(numa_gpu_bratu3d* op, const numa_gpu_vec* xpt, int jvp_mode,
                           numa_gpu_provider* provider, const numa_gpu_vec* b, numa_gpu_vec* x,
                           double rtol, size_t restart, size_t max_iters, int zero_guess,
                           int orth, int flexible, numa_gpu_krylov_space* save,
                           const numa_gpu_vec* r_init, numa_gmres_result* result);
/* gmres_recycled (linalg/gmres.hpp:229-323) with the Bratu3D Jacobian at xpt. */
int numa_gpu_gmres_recycled_bratu3d(numa_gpu_bratu3d* op, const numa_gpu_vec* xpt, int jvp_mode,
                                    numa_gpu_provider* provider, const numa_gpu_vec* b,
                                    numa_gpu_vec* x, double rtol, size_t restart,
                                    size_t max_iters, int orth,
                                    const numa_gpu_krylov_space* space,
                                    numa_gpu_krylov_space* save, numa_gmres_result* result);

/* ---------------------------------------------------------------- nonlinear drivers */
/* Eisenstat-Walker forcing term, detail::forcing (krylov_newton.hpp:54-65); host arithmetic. */
double numa_gpu_forcing(const numa_krylov_params* p, size_t k, double rnorm, double rprev,
                        double eta_prev, double res0);
/* newton_krylov(f, x0, p, pc) (krylov_newton.hpp:69-114).  x holds x0 on entry and the final
 * iterate on return (KrylovResult::x).  provider may be NULL (NoPrecond). */
int numa_gpu_newton_krylov(numa_gpu_bratu3d* op, numa_gpu_vec* x, const numa_krylov_params* p,
                           numa_gpu_provider* provider, numa_krylov_result* result);
/* chebyshev_inexact(f, x0, p, pc) (krylov_newton.hpp:116-189); p->recycle selects recycling. */
int numa_gpu_chebyshev_inexact(numa_gpu_bratu3d* op, numa_gpu_vec* x, const numa_krylov_params* p,
                               numa_gpu_provider* provider, numa_krylov_result* result);
/* tf_chebyshev_2018(f, x0, p, pc) (methods/tf_chebyshev_2018.hpp:52-132). */
int numa_gpu_tf_chebyshev_2018(numa_gpu_bratu3d* op, numa_gpu_vec* x, const numa_krylov_params* p,
                               numa_gpu_provider* provider, numa_krylov_result* result);

/* The three drivers on a Burgers2D: method of numa_gpu_method (CHEB_REC sets p->recycle).
 * The same functions as above, templated in the reference on the operator type. */
int numa_gpu_burgers2d_solve(numa_gpu_burgers2d* op, int method, numa_gpu_vec* x,
                             const numa_krylov_params* p, numa_gpu_provider* provider,
                             numa_krylov_result* result);

/* One call from host buffers to host buffers: Bratu3D(n, lambda), provider of precond_kind
 * (NONE, POISSON_MG with pre = post = 2 and mg_precision, JACOBI, or JACOBIAN_MG: the FP32 V(2,2)
 * with Jacobian-aware coarse levels, mg_precision ignored), method of numa_gpu_method,
 * x0[n^3] -> x_out[n^3].
 * The shape of apps/smoke_bratu.cpp:125-148 and apps/run_campaign.cpp:344-390.  With
 * NUMA_GPU_METHOD_NK and page-locked buffers the transfers overlap the solve: a pinned x0 goes up
 * in plane pieces under the first residual evaluation, and the iterate predicted to be the last is
 * copied to a pinned x_out while its residual is evaluated.  Results do not depend on it. */
int numa_gpu_solve_bratu3d_host(numa_gpu_ctx* ctx, size_t n, double lambda, int method,
                                int precond_kind, int mg_precision, const numa_krylov_params* p,
                                const double* x0, double* x_out, numa_krylov_result* result);
/* The same for Burgers2D(n, nu, dt, amplitude), precond_kind NONE or BURGERS_MG, x0[2n^2] ->
 * x_out[2n^2] (apps/run_campaign.cpp:577-593). */
int numa_gpu_solve_burgers2d_host(numa_gpu_ctx* ctx, size_t n, double nu, double dt, double amplitude,
                                  int method, int precond_kind, const numa_krylov_params* p,
                                  const double* x0, double* x_out, numa_krylov_result* result);

/* ---------------------------------------------------------------- learned preconditioner */
/* No counterpart in the reference.  A 4-level 3D convolutional network on the multigrid hierarchy
 * (base grid n0 in {15, 31, 63}, then (n-1)/2 three times; 16/32 channels, ~0.22M parameters) that
 * maps three feature fields (residual, Jacobian coefficient, V-cycle output, restricted to n0^3) to
 * a correction; BF16 activations, convolutions and their input gradients on the tensor cores,
 * FP32 master weights.  Parameters are FP32, layer by layer: W[27][cin][cout] then b[cout]. */
int numa_gpu_learned_create(numa_gpu_ctx* ctx, size_t n0, uint64_t seed, numa_gpu_learned** out);
int numa_gpu_learned_destroy(numa_gpu_learned* net);
int numa_gpu_learned_num_params(const numa_gpu_learned* net, size_t* n);
int numa_gpu_learned_get_params(numa_gpu_learned* net, float* host, size_t n);
int numa_gpu_learned_set_params(numa_gpu_learned* net, const float* host, size_t n);
/* out[n0^3] = channel 0 of the network applied to features[n0^3][3] (host buffers). */
int numa_gpu_learned_forward(numa_gpu_learned* net, const float* features, float* out);
/* loss = mean (out - target)^2 and its gradient with respect to the parameters (host buffers). */
int numa_gpu_learned_gradient(numa_gpu_learned* net, const float* features, const float* target, float* loss,
                              float* grad);

/* Training on the GPU from residual-error pairs of GMG-preconditioned solves: for `instances`
 * seeded lambda ~ U[lambda_min, lambda_max], Bratu3D(n_fine, lambda) is solved (mixed
 * Newton-Krylov), and at the states u = s u*, s = 0, 1/(states-1), ..., 1, the Jacobian systems
 * J e = r are solved by FGMRES(30) + FP32 V-cycle to solve_rtol for r = F(u), the first
 * krylov_per_state Arnoldi vectors of that solve (the inputs FGMRES gives the preconditioner) and
 * rhs_per_state seeded sums of 8 Gaussian bumps.  With q = r - J V r (the residual one FP32
 * V-cycle leaves) the network learns R^l (e - V r) / rms(R^l q) from (R^l q / rms, R^l c / 10) on
 * the level l of the fine hierarchy whose grid is n0; Adam, gradients summed over a batch. */
typedef struct numa_learned_train_params {
    size_t n_fine;
    double lambda_min, lambda_max;
    int instances, states, rhs_per_state, krylov_per_state;
    int epochs, batch;
    float lr;
    uint64_t seed;
    double solve_rtol;
} numa_learned_train_params;
typedef struct numa_learned_train_report {
    size_t samples;
    double gen_seconds, train_seconds;
    float loss_first, loss_last;  /* mean loss per sample, first and last epoch */
    float target_ms;              /* mean squared target: the loss of predicting zero */
} numa_learned_train_report;
int numa_gpu_learned_train(numa_gpu_learned* net, const numa_learned_train_params* p,
                           numa_learned_train_report* report);
/* FGMRES preconditioner for Bratu3D(n) (odd n coarsening to the network's base grid): z = V(r) +
 * s P^l net(R^l q / s, R^l c / 10), q = r - J V(r), s = rms(R^l q), with the FP32 V-cycle and the
 * FP32 Jacobian product at the iterate the provider was made at (make needs the coefficient
 * lambda e^u, which the nonlinear drivers pass; the public make(x) has none); during one linear
 * solve it falls back to the plain V-cycle once an iteration reduces the residual by less than the
 * factor `stall` (e.g. 0.9).  Use with flexible = 1.  The network must outlive the provider. */
int numa_gpu_provider_create_learned(numa_gpu_ctx* ctx, size_t n, numa_gpu_learned* net, double stall,
                                     numa_gpu_provider** out);
/* Network applications and fallbacks of a learned provider since its creation. */
int numa_gpu_provider_learned_stats(numa_gpu_provider* p, size_t* applies, size_t* fallbacks);

/* ---------------------------------------------------------------- Brusselator1DStep */
/* Brusselator1DStep(n, dt) (problems/brusselator1d.hpp:22-45): one implicit-Euler step of the 1D
 * Brusselator, A = 1, B = 3, alpha = 1/50, Dirichlet u = 1, v = 3; N = 2n, w = (u, v). */
int numa_gpu_brusselator1d_create(numa_gpu_ctx* ctx, size_t n, double dt, numa_gpu_brusselator1d** out);
int numa_gpu_brusselator1d_destroy(numa_gpu_brusselator1d* op);
int numa_gpu_brusselator1d_size(const numa_gpu_brusselator1d* op, size_t* N);
/* out = previous time level u = 1 + sin(2 pi x), v = 3     Brusselator1DStep::previous (:44) */
int numa_gpu_brusselator1d_previous(numa_gpu_brusselator1d* op, numa_gpu_vec* out);
/* out = F(w)                                               Brusselator1DStep::eval (:47-69) */
int numa_gpu_brusselator1d_eval(numa_gpu_brusselator1d* op, const numa_gpu_vec* w, numa_gpu_vec* out);
/* out = F'(w) d   mode ANALYTIC: jvp (:71-98); FD: jvp_fd */
int numa_gpu_brusselator1d_jvp(numa_gpu_brusselator1d* op, const numa_gpu_vec* w, const numa_gpu_vec* d,
                               numa_gpu_vec* out, int mode);
/* out = F''(w)[d,d] mode ANALYTIC: d2 (:100-118); FD: d2_fd */
int numa_gpu_brusselator1d_d2(numa_gpu_brusselator1d* op, const numa_gpu_vec* w, const numa_gpu_vec* d,
                              numa_gpu_vec* out, int mode);
/* The drivers on a Brusselator1DStep (CHEB_REC sets p->recycle). */
int numa_gpu_brusselator1d_solve(numa_gpu_brusselator1d* op, int method, numa_gpu_vec* x,
                                 const numa_krylov_params* p, numa_gpu_provider* provider,
                                 numa_krylov_result* result);
/* BrusselatorJacobi{op} (:194-222): 2x2 point blocks at the Newton iterate. */
int numa_gpu_provider_create_brusselator_jacobi(numa_gpu_brusselator1d* op, numa_gpu_provider** out);
/* Host buffers: x0[2n] (NULL = previous(), run_campaign's natural start) -> x_out[2n];
 * precond_kind NONE or BRUSS_JACOBI. */
int numa_gpu_solve_brusselator1d_host(numa_gpu_ctx* ctx, size_t n, double dt, int method, int precond_kind,
                                      const numa_krylov_params* p, const double* x0, double* x_out,
                                      numa_krylov_result* result);

/* ---------------------------------------------------------------- Brusselator2D (periodic) */
/* Implicit-Euler step of the 2-species Brusselator on an n x n periodic grid of the unit square
 * (h = 1/n), the reaction terms of brusselator1d.hpp:4-10 with parameters A, B, D_u, D_v, dt:
 * F(w) = (w - w_prev)/dt - diag(D_u, D_v) Lap_h w - (A + u^2 v - (B+1) u, B u - u^2 v);
 * N = 2 n^2, w = (u, v) component-major, row-major planes.  The previous level starts at zero. */
int numa_gpu_brusselator2d_create(numa_gpu_ctx* ctx, size_t n, const numa_brusselator2d_params* p,
                                  numa_gpu_brusselator2d** out);
int numa_gpu_brusselator2d_destroy(numa_gpu_brusselator2d* op);
int numa_gpu_brusselator2d_size(const numa_gpu_brusselator2d* op, size_t* N);
int numa_gpu_brusselator2d_set_previous(numa_gpu_brusselator2d* op, const numa_gpu_vec* w);
int numa_gpu_brusselator2d_eval(numa_gpu_brusselator2d* op, const numa_gpu_vec* w, numa_gpu_vec* out);
int numa_gpu_brusselator2d_jvp(numa_gpu_brusselator2d* op, const numa_gpu_vec* w, const numa_gpu_vec* d,
                               numa_gpu_vec* out, int mode);
int numa_gpu_brusselator2d_d2(numa_gpu_brusselator2d* op, const numa_gpu_vec* w, const numa_gpu_vec* d,
                              numa_gpu_vec* out, int mode);
/* One nonlinear solve from x with the current previous level. */
int numa_gpu_brusselator2d_solve(numa_gpu_brusselator2d* op, int method, numa_gpu_vec* x,
                                 const numa_krylov_params* p, numa_gpu_provider* provider,
                                 numa_krylov_result* result);
/* `steps` implicit-Euler steps: each takes the state x as the previous level and the Newton start
 * and leaves its solution in x; results[steps] (may be NULL). */
int numa_gpu_brusselator2d_advance(numa_gpu_brusselator2d* op, int method, size_t steps, numa_gpu_vec* x,
                                   const numa_krylov_params* p, numa_gpu_provider* provider,
                                   numa_krylov_result* results);
/* Coupled-block periodic multigrid V(pre, post) bound at each Newton iterate; precision FP64 or FP32. */
int numa_gpu_provider_create_brusselator_mg(numa_gpu_brusselator2d* op, int precision, int pre, int post,
                                            numa_gpu_provider** out);
/* Host buffers: x0[2n^2] -> x_out[2n^2] after `steps` steps; precond_kind NONE or BRUSS_MG with
 * V(2,2) in mg_precision.  Operator, provider and state are kept in the context between calls. */
int numa_gpu_brusselator2d_advance_host(numa_gpu_ctx* ctx, size_t n, const numa_brusselator2d_params* p,
                                        size_t steps, int method, int precond_kind, int mg_precision,
                                        const numa_krylov_params* kp, const double* x0, double* x_out,
                                        numa_krylov_result* results);
/* The multigrid alone: levels halve an even n while the coarse n is even and >= 4. */
int numa_gpu_bmg2d_create(numa_gpu_ctx* ctx, size_t n, const numa_brusselator2d_params* p, int precision, int pre,
                          int post, numa_gpu_bmg2d** out);
int numa_gpu_bmg2d_destroy(numa_gpu_bmg2d* mg);
int numa_gpu_bmg2d_levels(const numa_gpu_bmg2d* mg, size_t* levels);
/* blocks K(w) of the Jacobian at the state w[2 n^2] */
int numa_gpu_bmg2d_set_state(numa_gpu_bmg2d* mg, const numa_gpu_vec* w);
/* z = V-cycle(r) */
int numa_gpu_bmg2d_apply(numa_gpu_bmg2d* mg, const numa_gpu_vec* r, numa_gpu_vec* z);

/* ---------------------------------------------------------------- batched solves */
/* No counterpart in the reference.  Solves Bratu3D(inst[i].n, inst[i].lambda) from u0 = 0 for every
 * instance with `method` and a PoissonMG V(2,2) provider of mg_precision, concurrently: `workers`
 * host threads, each with its own context and stream on `device`, take instances largest first;
 * operators, hierarchies and workspaces are kept per grid size and reused.  results[i] holds the
 * counts of instance i; *wall_seconds the wall time of the whole batch (including the first use
 * of each grid size on each worker). */
typedef struct numa_batch_instance {
    size_t n;
    double lambda;
} numa_batch_instance;
typedef struct numa_batch_result {
    int32_t converged, status;
    uint64_t iters, n_F, n_JVP, n_lin_iters, n_prec;
    double res_rel, seconds;
} numa_batch_result;
int numa_gpu_solve_batch(int device, const numa_batch_instance* inst, size_t count, int method, int mg_precision,
                         const numa_krylov_params* p, int workers, numa_batch_result* results,
                         double* wall_seconds);
/* The same with the workers' device state (contexts, operators, hierarchies, workspaces) kept
 * between calls: create once, solve many batches, destroy. */
typedef struct numa_gpu_batch numa_gpu_batch;
int numa_gpu_batch_create(int device, int workers, numa_gpu_batch** out);
int numa_gpu_batch_destroy(numa_gpu_batch* b);
/* How many of the executor's workers a batch uses (1 ... the count given at creation). */
int numa_gpu_batch_set_workers(numa_gpu_batch* b, int workers);
/* Schedule autotuner: for each candidate worker count, one untimed and one timed batch of these
 * instances; the fastest becomes the executor's worker count (*chosen); seconds[c] (may be NULL)
 * the timed batch of candidate c. */
int numa_gpu_batch_autotune(numa_gpu_batch* b, const numa_batch_instance* inst, size_t count, int method,
                            int mg_precision, const numa_krylov_params* p, const int* candidates, int ncand,
                            int* chosen, double* seconds);
int numa_gpu_batch_solve(numa_gpu_batch* b, const numa_batch_instance* inst, size_t count, int method,
                         int mg_precision, const numa_krylov_params* p, numa_batch_result* results,
                         double* wall_seconds);
/* Message of the last failing batched call in this process ("" if it succeeded). */
const char* numa_gpu_batch_last_error(void);

/* Batched solves in one set of launches (no counterpart in the reference, whose campaign runner
 * solves instances one after another, apps/run_campaign.cpp:344-475): every instance advances
 * through newton_krylov (methods/krylov_newton.hpp:69-114) in lockstep, FGMRES(restart) with the
 * mixed path's FP32 basis and one-pass classical Gram-Schmidt, right-preconditioned by the FP32
 * V(2,2) multigrid cycle, FP32 Jacobian products, FP64 residual, update and least squares.  One
 * kernel launch per operation covers all instances (a packed instance table; the multigrid levels
 * of one size from all instances in one launch); every scalar decision (forcing term, Givens
 * rotations, restart, Armijo line search, convergence) is taken on the device per instance; each
 * Arnoldi step and each line-search trial is a captured CUDA graph.  Grid sizes n = 2^k - 1 with
 * 31 <= n <= 1023; u0 = 0.  Created on a context (its stream and device); the packed vectors, the
 * Krylov basis and the multigrid pools stay allocated until destroy. */
typedef struct numa_gpu_bsolver numa_gpu_bsolver;
typedef struct numa_batch_tuning {
    int32_t planes;          /* planes a thread marches in the residual and Jacobian stencils */
    int32_t elems_per_block; /* elements a block of the element-wise passes covers */
    int32_t reserved[6];
} numa_batch_tuning;
int numa_gpu_bsolver_create(numa_gpu_ctx* ctx, const numa_batch_instance* inst, size_t count,
                            const numa_krylov_params* p, numa_gpu_bsolver** out);
int numa_gpu_bsolver_destroy(numa_gpu_bsolver* s);
/* Solves every instance from u0 = 0.  results[i] for inst[i]; x_out (may be NULL): host buffer of
 * sum n_i^3 doubles receiving the solutions packed in the order of inst; seconds (may be NULL):
 * wall time of the call. */
int numa_gpu_bsolver_solve(numa_gpu_bsolver* s, double* x_out, numa_batch_result* results, double* seconds);
int numa_gpu_bsolver_get_tuning(const numa_gpu_bsolver* s, numa_batch_tuning* t);
int numa_gpu_bsolver_set_tuning(numa_gpu_bsolver* s, const numa_batch_tuning* t);
/* Tile-shape autotuner: one warm and one timed batch for each (planes[a], elems[b]) pair, the
 * fastest kept and returned in *chosen; seconds[a * ne + b] (may be NULL) = the timed batch. */
int numa_gpu_bsolver_autotune(numa_gpu_bsolver* s, const int* planes, int np, const int* elems, int ne,
                              numa_batch_tuning* chosen, double* seconds);

/* ---------------------------------------------------------------- V-cycle without allocation */
/* No counterpart in the reference.  For callers that cannot allocate device memory when they
 * apply the preconditioner: another library's solver callback that must not allocate or free on
 * every application (cudaMalloc / cudaFree can synchronise the device), or a program whose
 * device-memory budget is fixed up front.  One FP64 V-cycle z = M^-1 r of PoissonMG(n, pre, post)
 * on grids up to 63^3, bit-identical to numa_gpu_mg_apply, with every work array in one static
 * device array of NUMA_GPU_NOALLOC_MAX_DOUBLES doubles (4.8 MB, held by each GPU that loads the
 * library until the process exits).  r and z are distinct device arrays of n^3 doubles on the
 * current device; the work is enqueued on `stream` (a cudaStream_t, NULL for the default stream)
 * and the call returns without waiting.  It calls no cudaMalloc, cudaFree or allocating library
 * routine.  Every call not under stream capture resolves the array's address with
 * cudaGetSymbolAddress (the first on a device may load the module) and keeps it for the device; a
 * call being captured into a CUDA graph uses the kept address and makes no call that capture
 * forbids.  So make one uncaptured call, in the context the graph will run in, before capturing;
 * graphs captured before a cudaDeviceReset or a change of context must be captured again.  The
 * iterates of the levels are cleared with cudaMemsetAsync when pre = 0 (a memset node in a
 * captured graph).  Every call shares the array,
 * so calls that may run concurrently on the GPU race: order them on one stream.  Returns
 * NUMA_GPU_ERR_TOO_LARGE when the hierarchy of n does not fit the array, and NUMA_GPU_ERR_CUDA,
 * leaving the error pending, when a CUDA error was already pending on entry. */
#define NUMA_GPU_NOALLOC_MAX_DOUBLES 600832
int numa_gpu_mg_apply_noalloc(size_t n, int pre, int post, const double* r, double* z, void* stream);

/* ---------------------------------------------------------------- diagnostics */
/* No counterpart in the reference: measurements for roofline reports.
 * FP64 FMA throughput of the context's GPU in TFLOP/s (eight independent FMA chains per thread). */
int numa_gpu_diag_fp64_peak(numa_gpu_ctx* ctx, double* tflops);
/* Average duration in ms of one red-black Gauss-Seidel colour pass on the finest level of mg
 * (the V-cycle's dominant kernel), over reps back-to-back launches timed with CUDA events. */
int numa_gpu_diag_time_smoother(numa_gpu_mg* mg, int reps, double* ms_per_pass);
/* Average duration in ms of one Bratu3D residual evaluation F(x) with its fused norm and the cache
 * the nonlinear drivers keep (c = lambda e^x; precision NUMA_GPU_FP32 adds RN32(c) and RN32(F), as
 * on the mixed path), over reps back-to-back launches timed with CUDA events. */
int numa_gpu_diag_time_eval(numa_gpu_bratu3d* op, const numa_gpu_vec* x, int precision, int reps,
                            double* ms_per_eval);
/* out = F(x) and *norm (may be NULL) = ||F(x)|| as the drivers' residual evaluation at that precision
 * forms them: FP64 as numa_gpu_bratu3d_eval; FP32 the mixed path's evaluation (FP64 result, its
 * 7-point sum in 64-bit fixed point rounded once, 6u - sum - lambda e^u with one rounding). */
int numa_gpu_diag_eval(numa_gpu_bratu3d* op, const numa_gpu_vec* x, int precision, numa_gpu_vec* out,
                       double* norm);
/* The same for the finest level of a Brusselator2D multigrid (its blocks must have been set). */
int numa_gpu_diag_time_bmg2d_pass(numa_gpu_bmg2d* mg, int reps, double* ms_per_pass);
/* out = e^x as the residual kernels compute it (Tang's table-driven method, FP64); cuda_ref
 * (may be NULL) = CUDA's exp(x).  For accuracy checks of the exponential. */
int numa_gpu_diag_exp(const numa_gpu_vec* x, numa_gpu_vec* out, numa_gpu_vec* cuda_ref);
/* out = a / b as the finite-difference quotients compute it: from RN(1/b) with Markstein's
 * correction, the IEEE division outside the safe exponent range.  out may alias a. */
int numa_gpu_diag_div(const numa_gpu_vec* a, double b, numa_gpu_vec* out);
/* One 3x3x3 convolution of the learned preconditioner on the tensor cores (tcgen05, BF16 operands,
 * FP32 accumulation), host buffers in and out, zero padding: y[v][co] = bias[co] +
 * sum_{tap, ci} x[v + tap][ci] w[tap][ci][co] on an n^3 grid (n <= 63), x channel-last [n^3][cin],
 * w [27][cin][cout] with tap = (dz*3 + dy)*3 + dx, offsets d - 1.  adjoint = 1 runs the
 * convolution with the reversed, transposed kernel (the gradient with respect to the input):
 * x is then [n^3][cout] and y [n^3][cin].  cin, cout in {16, 32}; bias may be NULL. */
int numa_gpu_diag_conv3d(numa_gpu_ctx* ctx, size_t n, int cin, int cout, int adjoint, const float* x,
                         const float* w, const float* bias, float* y);
/* The learned preconditioner's weight and bias gradients of one 3x3x3 convolution on the tensor
 * cores (tcgen05, BF16 operands, FP32 accumulation), host buffers: dw[tap][ci][co] = sum_v
 * x[v + tap][ci] g[v][co] over the n^3 grid (zero outside), db[co] = sum_v g[v][co]; x [n^3][cin],
 * g [n^3][cout], n <= 63, cin, cout in {16, 32}. */
int numa_gpu_diag_conv3d_wgrad(numa_gpu_ctx* ctx, size_t n, int cin, int cout, const float* x, const float* g,
                               float* dw, float* db);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* NUMA_GPU_H */
