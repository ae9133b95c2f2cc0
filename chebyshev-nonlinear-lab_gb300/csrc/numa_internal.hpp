// numa_internal.hpp — internal C++ interfaces of libnuma_gpu (device pointers throughout).
//
// The classes mirror the reference's C++20 objects (namespace numa::op): Bratu3D, PoissonMG,
// the preconditioner providers, gmres / gmres_recycled and the nonlinear drivers.  They hold
// device memory and launch the CUDA kernels of the .cu files beside this header; the C ABI in
// capi.cu wraps them.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

#include "common.cuh"

namespace numa::gpu {

// ------------------------------------------------------------------------------ BLAS-1
// operators/operator.hpp:19-41.  Results land in device memory (out may be a scalar slot).
void dev_dot(Context& ctx, const double* a, const double* b, size_t N, double* out);
void dev_norm2(Context& ctx, const double* a, size_t N, double* out);
void dev_axpy(Context& ctx, double a, const double* x, double* y, size_t N);
void dev_fill(Context& ctx, double* y, double value, size_t N);
void dev_copy(Context& ctx, const double* src, double* dst, size_t N);
// xn = x - lam * z (krylov_newton.hpp:99, :173)
void dev_newton_step(Context& ctx, const double* x, const double* z, double lam, double* xn, size_t N);
// xn = x - z - 0.5 u (krylov_newton.hpp:166)
void dev_cheb_step(Context& ctx, const double* x, const double* z, const double* u, double* xn, size_t N);
// y = -y (tf_chebyshev_2018.hpp:95-96) and y = -0.5 y (:100-102)
void dev_scale_inplace(Context& ctx, double* y, double a, size_t N);

// ------------------------------------------------------------------------------ Bratu3D
struct SolverWorkspace;

class Bratu3D {
public:
    Bratu3D(Context& ctx, size_t n, double lambda);
    ~Bratu3D();
    // Device work arrays of the nonlinear drivers for this operator, kept between solves so
    // that a solve allocates nothing after the first (created on first use).
    SolverWorkspace& workspace();
    size_t size() const { return N_; }
    size_t grid() const { return n_; }
    double lambda() const { return lambda_; }
    double h2inv() const { return h2inv_; }
    Context& ctx() { return ctx_; }

    // out = F(x).  Optional: c_out = lambda e^x (the Jacobian coefficient at x) and
    // norm_out = ||F(x)|| (device scalar).  bratu3d.hpp:21-31
    void eval(const double* x, double* out, double* c_out = nullptr, double* norm_out = nullptr);
    // c = lambda e^x
    void coef(const double* x, double* c);
    // out = F'(x) v with the coefficient c = lambda e^x already formed (bratu3d.hpp:33-43).
    void jvp_c(const double* c, const double* v, double* out);
    // Mixed precision: the same with FP32 arithmetic (c32 = RN32(c)), FP64 in and out.
    void jvp_c32(const float* c32, const double* v, double* out);
    void coef32(const double* c, float* c32);
    // out = F'(x) v computing e^x in the kernel.
    void jvp_x(const double* x, const double* v, double* out);
    // out = F''(x)[v,v] = -c v^2 (bratu3d.hpp:46-56).
    void d2_c(const double* c, const double* v, double* out);
    // d = 6 h^-2 - c (bratu3d.hpp:59-69).
    void jacobi_diag_c(const double* c, double* d);

    // Finite-difference forms of operators/operator.hpp:101-134.  f0 = F(x) must be supplied
    // (it is the same vector the reference recomputes inside the call); xnorm = ||x|| as a
    // device scalar.  Scratch vectors come from the object.
    void jvp_fd(const double* x, const double* f0, const double* xnorm_dev, const double* v, double* out);
    void d2_fd(const double* x, const double* f0, const double* xnorm_dev, const double* v, double* out);

private:
    Context& ctx_;
    size_t n_, N_;
    double lambda_, h2inv_;
    DeviceArray<double> s1_, s2_, s3_;  // FD scratch
    std::unique_ptr<SolverWorkspace> ws_;
};

// ------------------------------------------------------------------------------ PoissonMG
class PoissonMG {
public:
    PoissonMG(Context& ctx, size_t n, int pre, int post, int precision, int max_levels);
    ~PoissonMG();
    size_t levels() const { return levels_.size(); }
    size_t size() const { return N0_; }
    int precision() const { return precision_; }
    // z = V-cycle(r); r and z are FP64 device vectors of size n^3 (poisson_mg.hpp:69-80).
    void apply(const double* r, double* z);
    // Diagnostic: average time (ms) of one red-black colour pass on the finest level, timed with
    // CUDA events over `reps` back-to-back passes on the context stream.
    double time_finest_pass(int reps);

    struct Level;

private:
    template <class T> void cycle(size_t l);
    void cycle32(size_t l);
    // The levels below the finest touch only the hierarchy's own arrays, so their part of the
    // cycle is captured once into a CUDA graph and replayed (one launch instead of ~10 a level).
    void coarse_cycle();
    Context& ctx_;
    cudaGraphExec_t coarse_exec_ = nullptr;
    uint64_t coarse_kernels_ = 0;
    // Finest-level arrays of the cycle in progress (the FP64 cycle works in the caller's r and z).
    void* x0_ = nullptr;
    const void* b0_ = nullptr;
    void* bs0_ = nullptr;
    double* z0_ = nullptr;  // FP32 cycle: FP64 output written by the last sweep of level 0
    size_t N0_;
    int pre_, post_, precision_;
    std::vector<std::unique_ptr<Level>> levels_;
    DeviceArray<double> scratch_r_;   // residual of the level being restricted (FP64 or FP32 bytes)
    DeviceArray<double> alias_b_;     // copy of r when r and z alias
};

// ------------------------------------------------------------------------------ providers
// Provider::make(x) -> Bound; Bound(r, z) (krylov_newton.hpp:20-22).
class Provider {
public:
    virtual ~Provider() = default;
    // Binds at the nonlinear iterate x; c = lambda e^x when the caller has it (may be null).
    virtual void make(const double* x, const double* c) = 0;
    virtual void apply(const double* r, double* z) = 0;
    virtual int kind() const = 0;
};

std::unique_ptr<Provider> make_identity_provider(Context& ctx, size_t N);
std::unique_ptr<Provider> make_mg_provider(Context& ctx, size_t n, int pre, int post, int precision,
                                           int max_levels);
std::unique_ptr<Provider> make_jacobi_provider(Bratu3D& op);

// ------------------------------------------------------------------------------ GMRES
struct GmresResult {
    size_t iters = 0, matvecs = 0, precs = 0;
    double rel_res = 0.0;
    bool converged = false, breakdown = false;
};

// Arnoldi basis of the last cycle (gmres.hpp:25-35).  V holds (at least) k+1 device vectors.
struct KrylovSpace {
    DeviceArray<double> V;
    size_t N = 0;
    size_t k = 0;
    std::vector<std::vector<double>> Hbar;  // (k+1) x k, host
    void clear() { k = 0; Hbar.clear(); }
};

// A linear operator / preconditioner on device vectors.
struct LinearOp {
    virtual ~LinearOp() = default;
    virtual void apply(const double* v, double* out) = 0;
};
struct Precond {
    virtual ~Precond() = default;
    virtual void apply(const double* r, double* z) = 0;
};

struct GmresOptions {
    double rtol = 1e-8;
    size_t restart = 50;
    size_t max_iters = 500;
    bool zero_guess = true;
    int orth = NUMA_GPU_ORTH_MGS;
    bool flexible = false;
};

class Gmres {
public:
    Gmres(Context& ctx, size_t N);
    // gmres (linalg/gmres.hpp:61-223).  M may be null (IdentityPrecond).
    GmresResult solve(LinearOp& A, Precond* M, const double* b, double* x, const GmresOptions& o,
                      KrylovSpace* save = nullptr, const double* r_init = nullptr);
    // gmres_recycled (linalg/gmres.hpp:229-323).
    GmresResult solve_recycled(LinearOp& A, Precond* M, const double* b, double* x,
                               const GmresOptions& o, const KrylovSpace& space,
                               KrylovSpace* save = nullptr);

private:
    void arnoldi_mgs(size_t j, double* w);
    void arnoldi_cgs2(size_t j, double* w);
    void precond_apply(Precond* M, const double* r, double* z);
    Context& ctx_;
    size_t N_;
    DeviceArray<double> V_, Z_, w_, r_, comb_, z_, rrec_;
    PinnedBuf pin_;
};

// Persistent arrays of a nonlinear solve (see Bratu3D::workspace).
struct SolverWorkspace {
    explicit SolverWorkspace(Context& ctx, size_t N) : gmres(ctx, N) {}
    DeviceArray<double> xb, Fa, Fb, ca, cb, z, u, w, scratch, xnorm;
    DeviceArray<float> c32;
    Gmres gmres;
    KrylovSpace space;
};

// ------------------------------------------------------------------------------ drivers
struct KrylovParams {
    double rtol_nl = 1e-8;
    size_t max_nl = 50;
    double eta_init = 0.5, eta_max = 0.9, gamma = 0.9, alpha = 2.0;
    double eta2_factor = 10.0, eta2_max = 0.5;
    size_t restart = 50, max_iters = 500;
    double armijo = 1e-4, min_lambda = 1e-4;
    bool recycle = false;
    int jvp_mode = 0, d2_mode = 0, orth = 0, jvp_precision = 0;
    bool flexible = false;
};

KrylovParams params_from_c(const numa_krylov_params* p);
double diag_fp64_peak_tflops(Context& ctx);
double forcing(const KrylovParams& p, size_t k, double rnorm, double rprev, double eta_prev, double res0);

// x holds x0 on entry and the final iterate on return.
void newton_krylov(Bratu3D& f, double* x, const KrylovParams& p, Provider* pc, numa_krylov_result& out);
void chebyshev_inexact(Bratu3D& f, double* x, const KrylovParams& p, Provider* pc, numa_krylov_result& out);
void tf_chebyshev_2018(Bratu3D& f, double* x, const KrylovParams& p, Provider* pc, numa_krylov_result& out);

}  // namespace numa::gpu
