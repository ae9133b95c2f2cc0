// numa_internal.hpp — internal C++ interfaces of libnuma_gpu (device pointers throughout).
//
// The classes mirror the reference's C++20 objects (namespace numa::op): Bratu3D, PoissonMG,
// the preconditioner providers, gmres / gmres_recycled and the nonlinear drivers.  They hold
// device memory and launch the CUDA kernels of the .cu files beside this header; the C ABI in
// capi.cu wraps them.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <functional>
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

// ------------------------------------------------------------------------------ operators
struct SolverWorkspace;

// A nonlinear operator on the device: the GPU form of the reference's NonlinearOperator /
// SecondOrderOperator concepts (operators/operator.hpp:43-58), which the drivers run on.
class NonlinearOp {
public:
    explicit NonlinearOp(Context& ctx) : ctx_(ctx) {}
    virtual ~NonlinearOp();
    Context& ctx() { return ctx_; }
    virtual size_t size() const = 0;
    // Doubles of data an iterate keeps for the Jacobian at it (0: none).
    virtual size_t cache_size() const = 0;
    // Announces the precision the Jacobian products of the coming solve will use, before any
    // evaluation (an operator may then keep what that precision needs in the cache).
    virtual void prepare_cache(int precision) { (void)precision; }
    // The evaluation in pieces along the slowest index, so that an upload of x can overlap it:
    // piece c writes the outputs from element eval_piece_begin(c) on (up to the next piece's begin),
    // reads x below eval_piece_need(c), and stores the raw sum of squares of its F values at *sumsq.
    // eval_pieces() = 0: not available.
    virtual int eval_pieces() const { return 0; }
    virtual size_t eval_piece_begin(int c) const {
        (void)c;
        return 0;
    }
    virtual size_t eval_piece_need(int c) const {
        (void)c;
        return size();
    }
    virtual void eval_piece(const double* x, double* out, double* cache, int c, double* sumsq) {
        (void)x;
        (void)out;
        (void)cache;
        (void)c;
        (void)sumsq;
    }
    // RN32(F) written by the evaluation that filled cache, where the operator keeps it (else null)
    virtual const float* f32_of_cache(const double* cache) const {
        (void)cache;
        return nullptr;
    }
    // RN32 of the Jacobian coefficient in cache, where the operator keeps it (else null)
    virtual const float* coef32_of_cache(const double* cache) const {
        (void)cache;
        return nullptr;
    }
    // out = F(x); cache := the Jacobian data at x (when cache_size() > 0); norm_out := ||F(x)||
    // as a device scalar (optional).
    virtual void eval(const double* x, double* out, double* cache, double* norm_out) = 0;
    // Binds J(x) for jvp_bound: the iterate, its cache, and the precision of the product
    // (NUMA_GPU_FP32 where the operator has a mixed-precision product, else FP64).
    virtual void bind(const double* x, const double* cache, int precision) = 0;
    virtual void jvp_bound(const double* v, double* out) = 0;
    // out = F'(x) v at an arbitrary point (no cache).
    virtual void jvp_at(const double* x, const double* v, double* out) = 0;
    // out = F'(x) v in FP64 at an iterate with its cache (the cache lets an operator skip work).
    virtual void jvp_cached(const double* x, const double* cache, const double* v, double* out) {
        (void)cache;
        jvp_at(x, v, out);
    }
    // out = F''(x)[v, v] at an iterate with its cache.
    virtual void d2(const double* x, const double* cache, const double* v, double* out) = 0;
    // The bound product in FP32 from an FP32 v, where bind() selected an FP32 form (has_jvp32).
    virtual bool has_jvp32() const { return false; }
    virtual void jvp_bound32(const float* v32, double* out) {
        (void)v32;
        (void)out;
    }
    // The same product stored in FP32 (its arithmetic is FP32 already), where has_jvp32f().
    virtual bool has_jvp32f() const { return false; }
    virtual void jvp_bound32f(const float* v32, float* out32) {
        (void)v32;
        (void)out32;
    }
    // The bound product from an FP32 v to FP64 accuracy (FP64 out), where has_jvp32x(): for linear
    // tolerances below what FP32 arithmetic reaches.
    virtual bool has_jvp32x() const { return false; }
    virtual void jvp_bound32x(const float* v32, double* out) {
        (void)v32;
        (void)out;
    }
    // The same product to FP32 accuracy with FP32 output (for an FP32 Krylov basis; its error near
    // the final rounding's), where has_jvp32x().
    virtual void jvp_bound32xf(const float* v32, float* out32) {
        (void)v32;
        (void)out32;
    }

    // Finite-difference forms of operators/operator.hpp:101-134 over eval.  f0 = F(x) must be
    // supplied (the same vector the reference recomputes inside the call); xnorm = ||x|| as a
    // device scalar.
    void jvp_fd(const double* x, const double* f0, const double* xnorm_dev, const double* v, double* out);
    void d2_fd(const double* x, const double* f0, const double* xnorm_dev, const double* v, double* out);

    // Device work arrays of the nonlinear drivers for this operator, kept between solves so
    // that a solve allocates nothing after the first (created on first use).
    SolverWorkspace& workspace();

protected:
    Context& ctx_;

private:
    DeviceArray<double> fd1_, fd2_, fd3_;  // finite-difference scratch
    std::unique_ptr<SolverWorkspace> ws_;
};

// ------------------------------------------------------------------------------ Bratu3D
class Bratu3D : public NonlinearOp {
public:
    Bratu3D(Context& ctx, size_t n, double lambda);
    ~Bratu3D() override;
    size_t size() const override { return N_; }
    size_t grid() const { return n_; }
    double lambda() const { return lambda_; }
    double h2inv() const { return h2inv_; }
    // A new lambda for the same grid (rebuilds the lambda-scaled exp table on the stream).
    void set_lambda(double lambda);

    // NonlinearOp: the cache of an iterate x is c = lambda e^x; for FP32 products it also holds
    // RN32(c) (N floats after the N doubles), written by the evaluation itself.
    // mixed cache: c (FP64), then RN32(c) and RN32(F) (N floats each)
    size_t cache_size() const override { return mixed_cache_ ? N_ + 2 * ((N_ + 1) / 2) : N_; }
    const float* f32_of_cache(const double* cache) const override {
        return mixed_cache_ && cache ? reinterpret_cast<const float*>(cache + N_ + (N_ + 1) / 2) : nullptr;
    }
    const float* coef32_of_cache(const double* cache) const override {
        return mixed_cache_ && cache ? reinterpret_cast<const float*>(cache + N_) : nullptr;
    }
    void prepare_cache(int precision) override { mixed_cache_ = precision == NUMA_GPU_FP32; }
    void eval(const double* x, double* out, double* cache, double* norm_out) override;
    int eval_pieces() const override;
    size_t eval_piece_begin(int c) const override;
    size_t eval_piece_need(int c) const override;
    void eval_piece(const double* x, double* out, double* cache, int c, double* sumsq) override;
    void bind(const double* x, const double* cache, int precision) override;
    void jvp_bound(const double* v, double* out) override;
    bool has_jvp32() const override { return bound_precision_ == NUMA_GPU_FP32; }
    void jvp_bound32(const float* v32, double* out) override;
    bool has_jvp32f() const override { return bound_precision_ == NUMA_GPU_FP32; }
    void jvp_bound32f(const float* v32, float* out32) override;
    // h^-2 = (n + 1)^2 must be an FP32 integer (n < 4095) for the double-FP32 scaling
    bool has_jvp32x() const override { return bound_precision_ == NUMA_GPU_FP32 && bound_c_ && n_ < 4095; }
    void jvp_bound32x(const float* v32, double* out) override;
    void jvp_bound32xf(const float* v32, float* out32) override;
    void jvp_at(const double* x, const double* v, double* out) override { jvp_x(x, v, out); }
    void jvp_cached(const double*, const double* cache, const double* v, double* out) override {
        jvp_c(cache, v, out);
    }
    void d2(const double* x, const double* cache, const double* v, double* out) override { d2_c(cache, v, out); }

    // out = F(x) (bratu3d.hpp:21-31)
    void eval(const double* x, double* out) { eval(x, out, nullptr, nullptr); }
    // c = lambda e^x
    void coef(const double* x, double* c);
    // out = F'(x) v with the coefficient c = lambda e^x already formed (bratu3d.hpp:33-43).
    void jvp_c(const double* c, const double* v, double* out);
    // Mixed precision: the same with FP32 arithmetic (c32 = RN32(c)), FP64 in and out.
    void jvp_c32(const float* c32, const double* v, double* out);
    // The product of an FP32 v to FP64 accuracy (double-FP32 stencil, FP64 c), FP64 out; n < 4095.
    void jvp_c32x(const double* c, const float* v32, double* out);
    void coef32(const double* c, float* c32);
    // out = F'(x) v computing e^x in the kernel.
    void jvp_x(const double* x, const double* v, double* out);
    // out = F''(x)[v,v] = -c v^2 (bratu3d.hpp:46-56).
    void d2_c(const double* c, const double* v, double* out);
    // d = 6 h^-2 - c (bratu3d.hpp:59-69).
    void jacobi_diag_c(const double* c, double* d);
    // Average ms of one residual evaluation with its fused norm and the cache the drivers keep
    // (c = lambda e^x; with precision FP32 also RN32(c) and RN32(F)), reps launches back to back.
    double time_eval(const double* x, int precision, int reps);
    // out = F(x) and *norm_host = ||F(x)|| as the drivers' evaluation at that precision forms them
    // (FP32: the mixed path's evaluation, with its fixed-point 7-point sum).
    void eval_as(const double* x, int precision, double* out, double* norm_host);

private:
    size_t n_, N_;
    double lambda_, h2inv_;
    const double* bound_c_ = nullptr;
    const float* bound_c32_ = nullptr;
    int bound_precision_ = NUMA_GPU_FP64;
    bool mixed_cache_ = false;
    DeviceArray<float> c32_;
    bool lt_on_ = false;           // lambda e^u from the lambda-scaled exp table
    DeviceArray<double2> lt2_;     // its FP64 pairs
    DeviceArray<float2> ltf_;      // and their RN32
    void eval_launch(const double* x, double* out, double* c_out, double* norm_out, dim3 grid, int ichunk, int zoff,
                     int norm_raw);
};

void bratu_jvp32(Context& ctx, int n, double h2inv, const float* c32, const double* v, double* out);
void bratu_coef32(Context& ctx, const double* c, float* c32, size_t N);

// ------------------------------------------------------------------------------ Burgers2D
// One implicit-Euler step of 2D viscous Burgers with a manufactured root
// (problems/burgers2d.hpp:23-218): w = (u, v), 2 n^2 unknowns.
class Burgers2D : public NonlinearOp {
public:
    Burgers2D(Context& ctx, size_t n, double nu, double dt, double amplitude);
    size_t size() const override { return 2 * n_ * n_; }
    size_t grid() const { return n_; }
    double nu() const { return nu_; }
    double dt() const { return dt_; }
    const double* exact() const { return exact_.p; }
    double cell_reynolds() const { return std::abs(amp_) / (nu_ * (static_cast<double>(n_) + 1.0)); }
    size_t cache_size() const override { return 0; }
    void eval(const double* x, double* out, double* cache, double* norm_out) override;
    void bind(const double* x, const double*, int) override { bound_x_ = x; }
    void jvp_bound(const double* v, double* out) override { jvp_at(bound_x_, v, out); }
    void jvp_at(const double* x, const double* v, double* out) override;
    void d2(const double* x, const double* cache, const double* v, double* out) override;

private:
    size_t n_;
    double nu_, dt_, amp_;
    double inv2h_, invh2_, invdt_;
    DeviceArray<double> source_, exact_;
    const double* bound_x_ = nullptr;
};

// ------------------------------------------------------------------------------ Brusselator
// Brusselator1DStep (problems/brusselator1d.hpp:22-192): one implicit-Euler step of the 1D
// Brusselator, A = 1, B = 3, alpha = 1/50, Dirichlet u = 1, v = 3; w = (u, v), 2 n unknowns.
class Brusselator1D : public NonlinearOp {
public:
    static constexpr double kA = 1.0, kB = 3.0, kAlpha = 1.0 / 50.0;
    Brusselator1D(Context& ctx, size_t n, double dt);
    size_t size() const override { return 2 * n_; }
    size_t grid() const { return n_; }
    double dt() const { return dt_; }
    // the previous time level u = 1 + sin(2 pi x), v = 3 (the natural Newton start)
    const double* previous() const { return prev_.p; }
    size_t cache_size() const override { return 0; }
    void eval(const double* x, double* out, double* cache, double* norm_out) override;
    void bind(const double* x, const double*, int) override { bound_x_ = x; }
    void jvp_bound(const double* v, double* out) override { jvp_at(bound_x_, v, out); }
    void jvp_at(const double* x, const double* v, double* out) override;
    void d2(const double* x, const double* cache, const double* v, double* out) override;
    // the 2x2 point blocks at x as planes a11 | a12 | a21 | a22 (local_jacobi_blocks, :120-141)
    void blocks(const double* x, double* a);

private:
    size_t n_;
    double dt_, h_ = 0.0, h2inv_ = 0.0;
    DeviceArray<double> prev_;
    const double* bound_x_ = nullptr;
};

// z = block^-1 r per point (BrusselatorJacobi::Bound, brusselator1d.hpp:198-214).
void brusselator_block_apply(Context& ctx, const double* a, const double* r, double* z, size_t n);

// Implicit-Euler step of the 2-species Brusselator on an n x n periodic grid (h = 1/n):
// F(w) = (w - w_prev)/dt - diag(D_u, D_v) Lap_h w - (A + u^2 v - (B+1) u, B u - u^2 v).
class Brusselator2D : public NonlinearOp {
public:
    Brusselator2D(Context& ctx, size_t n, const numa_brusselator2d_params& p);
    size_t size() const override { return 2 * n_ * n_; }
    size_t grid() const { return n_; }
    const numa_brusselator2d_params& params() const { return P_; }
    const double* previous() const { return prev_.p; }
    void set_previous(const double* w);
    size_t cache_size() const override { return 0; }
    // FP32 products announced: the drivers' evaluations (with the norm) form the Laplacians in fixed point
    // (k_b2_eval FIXED); an evaluation without the norm keeps the FP64 differences
    void prepare_cache(int precision) override { fixed_sum_ = precision == NUMA_GPU_FP32; }
    void eval(const double* x, double* out, double* cache, double* norm_out) override;
    // FP32 binding: the coefficients (2uv, u^2) of the iterate in FP32; products in FP32 arithmetic
    void bind(const double* x, const double*, int precision) override;
    void jvp_bound(const double* v, double* out) override;
    bool has_jvp32() const override { return bound_precision_ == NUMA_GPU_FP32; }
    void jvp_bound32(const float* v32, double* out) override;
    bool has_jvp32f() const override { return bound_precision_ == NUMA_GPU_FP32; }
    void jvp_bound32f(const float* v32, float* out32) override;
    void jvp_at(const double* x, const double* v, double* out) override;
    void d2(const double* x, const double* cache, const double* v, double* out) override;

private:
    size_t n_;
    numa_brusselator2d_params P_;
    DeviceArray<double> prev_, coef32_;
    const double* bound_x_ = nullptr;
    int bound_precision_ = NUMA_GPU_FP64;
    bool fixed_sum_ = false;
};

// Periodic geometric multigrid V(pre, post) for the coupled 2x2-block Jacobian of Brusselator2D,
// K(w) - diag(D_u, D_v) Lap_h: levels halve n while the coarse n is even and >= 4, red-black
// point-block Gauss-Seidel, full weighting of residuals and blocks, bilinear periodic
// prolongation, 30 sweeps on the coarsest level; FP64 or FP32 level arrays.
class BrussMG2D {
public:
    BrussMG2D(Context& ctx, size_t n, const numa_brusselator2d_params& p, int precision, int pre, int post);
    ~BrussMG2D();
    size_t levels() const { return levels_.size(); }
    size_t size() const { return 2 * n0_ * n0_; }
    // blocks K at the state w (FP64 planes), restricted to every level
    void set_state(const double* w);
    // z = V-cycle(r), FP64 planes in and out
    void apply(const double* r, double* z);
    // z32 = V-cycle(r) in FP32 only, for an FP32 hierarchy with more than one level.
    bool supports_out32() const { return precision_ == NUMA_GPU_FP32 && levels_.size() > 1; }
    void apply32(const double* r, float* z32);
    // The same from an FP32 right-hand side (an FP32 Krylov basis vector), read as it is.
    void apply32f(const float* r32, float* z32);
    // ms of one finest-level colour pass (CUDA events, reps back-to-back launches)
    double time_finest_pass(int reps);
    struct Level;

private:
    template <class T> void cycle(size_t l);
    void coarse_cycle();
    Context& ctx_;
    size_t n0_;
    numa_brusselator2d_params P_;
    int precision_, pre_, post_;
    std::vector<std::unique_ptr<Level>> levels_;
    DeviceArray<double> alias_;
    const double* r0_ = nullptr;
    const float* r32_ = nullptr;  // FP32 right-hand side of the current apply32f
    double* z0_ = nullptr;
    float* z32_ = nullptr;
    cudaGraphExec_t coarse_exec_ = nullptr;
    uint64_t coarse_kernels_ = 0;
    bool state_set_ = false;
    int tail_first_ = -1;          // first level of the one-block tail (-1: none)
    int tail_count_ = 0;
    size_t tail_smem_ = 0;         // its shared memory in bytes
    DeviceArray<double> tail_desc_;  // its level descriptors
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
    // z32 = V-cycle(r) in FP32 only (the values apply() widens into z), where supports_out32().
    bool supports_out32() const;
    void apply32(const double* r, float* z32);
    // The same from an FP32 right-hand side (an FP32 Krylov basis vector), read as it is.
    void apply32f(const float* r32, float* z32);
    // Diagnostic: average time (ms) of one red-black colour pass on the finest level, timed with
    // CUDA events over `reps` back-to-back passes on the context stream.
    double time_finest_pass(int reps);
    // FP32 cycle: RN32(r) of the last apply on the finest level and its layout (colour-split when odd).
    const float* fine_b32() const;
    // Jacobian-aware coarse levels (FP32 cycle with a one-CTA tail): the levels n <= 15 then solve
    // with -Lap_h - c instead of -Lap_h, c the full-weighting restriction of the fine coefficient c
    // (for Bratu3D's Jacobian, c = lambda e^u) set by set_coarse_coefficient.
    bool supports_coarse_jacobian() const { return precision_ == NUMA_GPU_FP32 && tail_l_ != SIZE_MAX; }
    // c32_fine (may be null): RN32(c_fine), read instead of c_fine (the same values, half the bytes).
    void set_coarse_coefficient(const double* c_fine, const float* c32_fine = nullptr);
    void clear_coarse_coefficient() { coarse_jac_ = false; }

    struct Level;

private:
    template <class T> void cycle(size_t l);
    void cycle32(size_t l);
    bool first_fused32(size_t l) const;
    // FP32 cycle: levels from tail_l_ (n <= 15) down run in one CTA (k_mg_tail); SIZE_MAX = none.
    size_t tail_l_ = SIZE_MAX;
    size_t tail_smem_ = 0;
    void launch_tail32();
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
    float* z32_out_ = nullptr;        // FP32 output of the current apply32
    const float* in32_ = nullptr;     // FP32 right-hand side of the current apply32f
    DeviceArray<double> scratch_r_;   // residual of the level being restricted (FP64 or FP32 bytes)
    DeviceArray<double> alias_b_;     // copy of r when r and z alias
    bool coarse_jac_ = false;         // the tail solves with the coefficient below
    bool graph_jac_ = false;          // the mode the coarse-level graph was captured in
    DeviceArray<float> cl_;           // the restricted coefficient of every level below the finest
    std::vector<size_t> cl_off_;      // offsets of the levels' coefficients in cl_
};

// ------------------------------------------------------------------------------ HelmholtzMG2D
// 2D V-cycle for alpha I - nu Lap_h (linalg/helmholtz_mg2d.hpp:13-158), FP64, bit-exact.
class HelmholtzMG2D {
public:
    HelmholtzMG2D(Context& ctx, size_t n, double alpha, double nu, int pre, int post);
    ~HelmholtzMG2D();
    size_t levels() const { return levels_.size(); }
    size_t size() const { return N0_; }
    // z = V-cycle(r), n^2 FP64 device vectors (helmholtz_mg2d.hpp:36-42).
    void apply(const double* r, double* z);
    struct Level;

private:
    void cycle(size_t l);
    Context& ctx_;
    size_t N0_;
    double alpha_;
    int pre_, post_;
    std::vector<std::unique_ptr<Level>> levels_;
    DeviceArray<double> resid_, alias_;
    double* x0_ = nullptr;
    const double* b0_ = nullptr;
};

// ------------------------------------------------------------------------------ providers
// Provider::make(x) -> Bound; Bound(r, z) (krylov_newton.hpp:20-22).
class Provider {
public:
    virtual ~Provider() = default;
    // Binds at the nonlinear iterate x; cache = the operator's Jacobian data at x (for Bratu3D
    // c = lambda e^x) when the caller has it (may be null).
    virtual void make(const double* x, const double* cache) = 0;
    // The same where the operator also keeps RN32 of its coefficient (c32, not null).
    virtual void make_c32(const double* x, const double* cache, const float* c32) {
        (void)c32;
        make(x, cache);
    }
    virtual void apply(const double* r, double* z) = 0;
    virtual int kind() const = 0;
    virtual void progress(size_t iters, double rel_res) {
        (void)iters;
        (void)rel_res;
    }
    // z32 = M r in FP32 only (the values apply() would widen into z), where has_apply32().
    virtual bool has_apply32() const { return false; }
    virtual void apply32(const double* r, float* z32) {
        (void)r;
        (void)z32;
    }
    // z32 = M r32 from an FP32 r, where has_apply32f().
    virtual bool has_apply32f() const { return false; }
    virtual void apply32f(const float* r32, float* z32) {
        (void)r32;
        (void)z32;
    }
};

std::unique_ptr<Provider> make_identity_provider(Context& ctx, size_t N);
std::unique_ptr<Provider> make_mg_provider(Context& ctx, size_t n, int pre, int post, int precision,
                                           int max_levels);
// The FP32 V-cycle whose coarse levels (n <= 15) solve with the Jacobian -Lap_h - c of the iterate it
// is bound at (c from the operator's cache): a preconditioner for Bratu3D's J = -Lap_h - lambda e^u.
std::unique_ptr<Provider> make_jacobian_mg_provider(Context& ctx, size_t n, int pre, int post);
std::unique_ptr<Provider> make_jacobi_provider(Bratu3D& op);
// BurgersMGProvider (problems/burgers2d.hpp:220-246): the HelmholtzMG2D V-cycle of
// (1/dt) I - nu Lap_h applied to each component.
std::unique_ptr<Provider> make_burgers_mg_provider(Context& ctx, size_t n, double nu, double dt, int pre, int post);
// BrusselatorJacobi (problems/brusselator1d.hpp:194-222).
std::unique_ptr<Provider> make_bruss_jacobi_provider(Brusselator1D& op);
// BrussMG2D bound at each Newton iterate.
std::unique_ptr<Provider> make_bruss_mg_provider(Context& ctx, size_t n, const numa_brusselator2d_params& p,
                                                 int precision, int pre, int post);

// ------------------------------------------------------------------------------ GMRES
struct GmresResult {
    size_t iters = 0, matvecs = 0, precs = 0;
    double rel_res = 0.0;
    bool converged = false, breakdown = false;
    bool stepped = false;  // GmresOptions::x_step holds x_base - x for the returned x
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
    // out = A v from an FP32 v, where A has an FP32 form.
    virtual bool has_apply32() const { return false; }
    virtual void apply32(const float* v32, double* out) {
        (void)v32;
        (void)out;
    }
    // out32 = A v32 stored in FP32, where has_apply32f().
    virtual bool has_apply32f() const { return false; }
    virtual void apply32f(const float* v32, float* out32) {
        (void)v32;
        (void)out32;
    }
    // out = A v from an FP32 v to FP64 accuracy, where has_apply32x().
    virtual bool has_apply32x() const { return false; }
    virtual void apply32x(const float* v32, double* out) {
        (void)v32;
        (void)out;
    }
    // ... rounded once to FP32, where has_apply32x().
    virtual void apply32xf(const float* v32, float* out32) {
        (void)v32;
        (void)out32;
    }
};
struct Precond {
    virtual ~Precond() = default;
    virtual void apply(const double* r, double* z) = 0;
    // z32 = M r in FP32 only, where M has an FP32 output.
    virtual bool has_apply32() const { return false; }
    virtual void apply32(const double* r, float* z32) {
        (void)r;
        (void)z32;
    }
    // z32 = M r32 from an FP32 r (an FP32 Krylov basis vector), where has_apply32f().
    virtual bool has_apply32f() const { return false; }
    virtual void apply32f(const float* r32, float* z32) {
        (void)r32;
        (void)z32;
    }
    // Called by GMRES after each Arnoldi step with the iteration count of the solve and the relative
    // residual estimate (a preconditioner may change strategy on stagnation, as FGMRES allows).
    virtual void progress(size_t iters, double rel_res) {
        (void)iters;
        (void)rel_res;
    }
};

struct GmresOptions {
    double rtol = 1e-8;
    size_t restart = 50;
    size_t max_iters = 500;
    bool zero_guess = true;
    int orth = NUMA_GPU_ORTH_MGS;
    bool flexible = false;
    double bnorm = -1.0;  // ||b|| when the caller knows it (>= 0), used by the flexible CGS1 solver
    const float* b32 = nullptr;  // RN32(b) when the caller has it (the FP32 Arnoldi basis starts from it)
    // With FP32 preconditioned vectors and a linear tolerance below 1e-5: compute A z_j to FP64 accuracy
    // where the operator offers it (LinearOp::has_apply32x), rounded once to FP32 into an FP32 basis down
    // to a tolerance of 1e-6, kept in FP64 with an FP64 basis below
    bool precise_tight = false;
    // When given (a Newton driver): the solution update also writes x_step = x_base - x, the full
    // Newton step, and reports it in GmresResult::stepped if that update was the solve's last
    const double* x_base = nullptr;
    double* x_step = nullptr;
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
    void arnoldi_cgs1(size_t j, double* w);
    GmresResult solve_lazy(LinearOp& A, Precond* M, const double* b, double* x, const GmresOptions& o,
                           const double* r_init);
    void precond_apply(Precond* M, const double* r, double* z);
    Context& ctx_;
    size_t N_;
    DeviceArray<double> V_, Z_, w_, r_, comb_, z_, rrec_;
    DeviceArray<float> Z32_;  // FGMRES preconditioned vectors in FP32 (FP32 preconditioner and product)
    DeviceArray<float> V32_;  // FGMRES basis in FP32 (FP32 hand-off, loose linear tolerance)
    DeviceArray<float> W32_;  // its A z_j in FP32
    DeviceArray<float> P32_;  // double-FP32 partial sums of a Gram-Schmidt update over a long FP32 basis
    PinnedBuf pin_;
};

// Persistent arrays of a nonlinear solve (see NonlinearOp::workspace).
struct SolverWorkspace {
    explicit SolverWorkspace(Context& ctx, size_t N) : gmres(ctx, N) {}
    DeviceArray<double> xb, Fa, Fb, ca, cb, z, u, w, scratch, xnorm;
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
    bool jvp_tight = false;  // GmresOptions::precise_tight for the Newton and Chebyshev solves
    bool coarse_jacobian = false;  // batched solver: Jacobian-aware multigrid tail
};

KrylovParams params_from_c(const numa_krylov_params* p);
double diag_fp64_peak_tflops(Context& ctx);
// out = the library's e^x (exp_tang) of x; ref (optional) = CUDA's exp(x).
void diag_exp(Context& ctx, const double* x, double* out, double* ref, size_t N);
void diag_div(Context& ctx, const double* a, double b, double* out, size_t N);
// One tensor-core 3x3x3 convolution from host buffers (learned.cu): y = conv(x, W) + b, FP32
// channel-last in and out, BF16 operands; flip = the adjoint convolution (gradient with respect to
// the input, W of shape [27][cin][cout] used as [27][cout][cin] with the taps reversed).
void diag_conv3d_wgrad(Context& ctx, int n, int cin, int cout, const float* x_h, const float* g_h, float* dw_h,
                       float* db_h);
void diag_conv3d(Context& ctx, int n, int cin, int cout, int flip, const float* x_h, const float* w_h,
                 const float* b_h, float* y_h);

// The learned preconditioner's network (learned_net.cu).
class LearnedNet;
LearnedNet* learned_create(Context& ctx, int n0, uint64_t seed);
void learned_destroy(LearnedNet* net);
size_t learned_num_params(const LearnedNet& net);
int learned_n0(const LearnedNet& net);
void learned_get_params(const LearnedNet& net, float* host);
void learned_set_params(LearnedNet& net, const float* host);
void learned_forward_host(Context& ctx, LearnedNet& net, const float* feat, float* out);
void learned_grad_host(Context& ctx, LearnedNet& net, const float* feat, const float* target, float* loss,
                       float* grad);
void learned_train(Context& ctx, LearnedNet& net, const numa_learned_train_params& p, numa_learned_train_report& rep);
class Provider;
std::unique_ptr<Provider> make_learned_provider(Context& ctx, size_t n, LearnedNet& net, double stall);
void learned_provider_stats(Provider& p, size_t* applies, size_t* fallbacks);
double forcing(const KrylovParams& p, size_t k, double rnorm, double rprev, double eta_prev, double res0);

// Many independent Bratu3D solves on one device (batch.cu); results[i] for inst[i].
struct BatchWorker;
class BatchExecutor {
public:
    BatchExecutor(int device, int workers);
    ~BatchExecutor();
    int workers() const { return (int)workers_.size(); }
    // how many of the workers a batch uses (1 ... workers())
    int active() const { return active_; }
    void set_active(int w);
    void solve(const numa_batch_instance* inst, size_t count, int method, int mg_precision,
               const numa_krylov_params* params, numa_batch_result* results, double* wall_seconds);
    // The schedule autotuner: for each candidate worker count, one untimed batch (sets the workers
    // up) and one timed batch of these instances; keeps the fastest as the active count and returns it.
    int autotune(const numa_batch_instance* inst, size_t count, int method, int mg_precision,
                 const numa_krylov_params* params, const int* candidates, int ncand, double* seconds);

private:
    int device_;
    int active_;
    std::vector<std::unique_ptr<BatchWorker>> workers_;
};

// Tile shapes of the batched solver's kernels (batch_solver.cu), picked by its autotuner:
// planes a thread marches in the residual and Jacobian stencils, elements a block of the
// element-wise passes (Gram-Schmidt, solution update, line-search step) covers.
struct BatchTuning {
    int planes = 8;
    int elems_per_block = 16384;
};

// Many Bratu3D instances of uneven size (n = 2^k - 1, 31 ... 1023) and lambda solved together by
// the mixed Newton-Krylov path, one launch per operation over a packed instance table.
class BatchSolver {
public:
    BatchSolver(Context& ctx, const numa_batch_instance* inst, size_t count, const KrylovParams& p);
    ~BatchSolver();
    // u0 = 0 for every instance; x_out (may be null): the solutions, packed in the caller's order.
    void solve(double* x_out, numa_batch_result* results, double* seconds);
    size_t instances() const;
    size_t total_unknowns() const;
    BatchTuning tuning() const;
    void set_tuning(const BatchTuning& t);
    // One warm and one timed batch for every (planes[a], elems[b]) pair; keeps and returns the fastest.
    BatchTuning autotune(const int* planes, int np, const int* elems, int ne, double* seconds);

    struct Impl;

private:
    std::unique_ptr<Impl> impl_;
};

// x holds x0 on entry and the final iterate on return.
constexpr int kEvalPieces = 8;  // most pieces of an evaluation overlapped with an upload
// Pinned host buffers of a Newton solve.  `host` (the initial point) goes up in pieces on `copy` while the
// first evaluation runs on the pieces already there.  `host_out`, when set, receives a trial point the
// linear model predicts to be the last while its residual is evaluated; `fetched` reports that the
// returned solution is that copy (otherwise the caller downloads it).
struct HostUpload {
    const double* host = nullptr;
    double* host_out = nullptr;
    bool fetched = false;
    cudaStream_t copy = nullptr;
    cudaEvent_t start = nullptr;
    cudaEvent_t done[kEvalPieces] = {};
    cudaEvent_t fetch_start = nullptr, fetch_done = nullptr;
    ~HostUpload() {
        for (cudaEvent_t e : done)
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t e : {start, fetch_start, fetch_done})
            if (e) cudaEventDestroy(e);
        if (copy) cudaStreamDestroy(copy);
    }
};
void newton_krylov(NonlinearOp& f, double* x, const KrylovParams& p, Provider* pc, numa_krylov_result& out,
                   HostUpload* up = nullptr);
void chebyshev_inexact(NonlinearOp& f, double* x, const KrylovParams& p, Provider* pc, numa_krylov_result& out);
void tf_chebyshev_2018(NonlinearOp& f, double* x, const KrylovParams& p, Provider* pc, numa_krylov_result& out);

}  // namespace numa::gpu
