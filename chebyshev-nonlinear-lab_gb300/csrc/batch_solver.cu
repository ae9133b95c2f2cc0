// batch_solver.cu — many Bratu3D instances of uneven grid size and lambda solved together on one
// GPU (the batched configuration): Newton-Krylov (methods/krylov_newton.hpp:69-114) with flexible
// GMRES (linalg/gmres.hpp:61-223, the mixed path's lazily normalised FP32 basis and one-pass
// classical Gram-Schmidt) right-preconditioned by the FP32 multigrid V-cycle
// (linalg/poisson_mg.hpp), every instance in lockstep, one launch per operation over all of them.
//
// What runs where:
//  * every vector operation is a kernel over the packed instance table (batch_kernels.cuh);
//  * every scalar decision of the reference's drivers — the forcing term, the Arnoldi bookkeeping
//    and Givens rotations, the least-squares solve, the restart test, the Armijo line search, the
//    convergence test — runs on the device, one thread per instance, in the host code's FP64
//    arithmetic, and leaves per-instance activity flags that the next kernels read;
//  * each Arnoldi step (V-cycle, Jacobian product, Gram-Schmidt, reductions, rotations) and each
//    line-search trial (step, residual, reductions, acceptance) is captured once as a CUDA graph and
//    replayed; the host reads one status word per replay to learn whether any instance is still
//    active, so every loop is bounded by the reference's own limits (max_nl, the restart length,
//    gmres_max_iters, min_lambda).
// Instances are independent: the same instance solved alone by the single-instance mixed path
// takes the same decisions up to the order of its reductions.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>

#include "batch_kernels.cuh"

namespace numa::gpu {
namespace {

// The per-instance scalar kernels, like every kernel here, are launched with programmatic stream
// serialisation and begin with pdl_wait(): they read what the previous kernel wrote.
constexpr int kScalarThreads = 128;
enum BFlag { kFlagNL = 1, kFlagLin = 2, kFlagRestart = 4, kFlagLS = 8 };

// Per-instance solver state on the device (arrays of length I unless a stride is given).
struct BState {
    int I, m;
    // flags and counters
    int *nl_act, *cur, *lin_act, *ls_act, *rs_act, *in_cyc, *assign, *lin_conv, *brk, *eval, *cmb, *conv;
    int *iters, *nF, *nJVP, *nlin, *nlinfail, *nprec, *lit, *lmv, *lpc;
    // scalars
    double *res0, *rnorm, *rprev, *eta_prev, *eta, *alpha, *bnorm, *fn2, *beta2, *inv_beta;
    // least squares (strides m + 1 for g, m for cs / sn / y, (m + 1) m for H)
    double *H, *cs, *sn, *g, *y;
    int* flags;
};

struct BParams {
    double rtol_nl, eta_init, eta_max, gamma, alpha, armijo, min_lambda;
    int max_iters;
};

// Eisenstat-Walker choice 2 with Kelley's safeguard and the oversolve floor (krylov_newton.hpp:54-65),
// the host forcing() in the same operations.
__device__ double bforcing(const BParams& p, int k, double rnorm, double rprev, double eta_prev, double res0) {
    if (k == 0) return p.eta_init;
    double eta = p.gamma * pow(rnorm / rprev, p.alpha);
    const double safe = p.gamma * pow(eta_prev, p.alpha);
    if (safe > 0.1) eta = fmax(eta, safe);
    eta = fmin(eta, p.eta_max);
    eta = fmax(eta, 0.5 * p.rtol_nl * res0 / rnorm);
    return fmin(eta, p.eta_max);
}

__global__ void k_binit(BState S) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.I) return;
    S.nl_act[t] = 1;
    S.cur[t] = 0;
    S.eval[t] = 1;
    S.lin_act[t] = S.ls_act[t] = S.rs_act[t] = S.in_cyc[t] = S.assign[t] = S.lin_conv[t] = S.brk[t] = 0;
    S.cmb[t] = S.conv[t] = 0;
    S.iters[t] = S.nF[t] = S.nJVP[t] = S.nlin[t] = S.nlinfail[t] = S.nprec[t] = 0;
    S.lit[t] = S.lmv[t] = S.lpc[t] = 0;
}

// after the first residual evaluation (krylov_newton.hpp:76-79)
__global__ void k_bfirst(BState S, BParams p) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.I) return;
    const double r = __dsqrt_rn(S.fn2[t]);
    S.rnorm[t] = r;
    S.res0[t] = r;
    S.rprev[t] = r;
    S.eta_prev[t] = p.eta_init;
    S.nF[t] = 1;
    S.eval[t] = 0;
}

// Newton iteration k of every active instance: the convergence test, the forcing term and the
// start of its FGMRES solve J z = F (zero first guess, u_0 = RN32(F) with sigma_0 = 1/||F||).
__global__ void k_bnl_begin(BState S, BParams p, BKry K, int k) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.I || !S.nl_act[t]) return;
    const double rnorm = S.rnorm[t];
    if (rnorm <= p.rtol_nl * S.res0[t]) {
        S.conv[t] = 1;
        S.nl_act[t] = 0;
        return;
    }
    const double eta = bforcing(p, k, rnorm, S.rprev[t], S.eta_prev[t], S.res0[t]);
    S.eta[t] = eta;
    S.in_cyc[t] = 1;
    S.lin_act[t] = 1;
    S.assign[t] = 1;
    S.lin_conv[t] = 0;
    S.brk[t] = 0;
    S.lit[t] = S.lmv[t] = S.lpc[t] = 0;
    S.bnorm[t] = rnorm;
    double* g = S.g + (long long)t * (S.m + 1);
    g[0] = rnorm;
    for (int i = 1; i <= S.m; ++i) g[i] = 0.0;
    K.sig[(long long)t * K.m1] = 1.0 / rnorm;
    K.sig2[(long long)t * K.m1] = 1.0 / (rnorm * rnorm);
    K.kdone[t] = 0;
    atomicOr(S.flags, kFlagNL | kFlagLin);
}

// The host bookkeeping of one Arnoldi step j (gmres.hpp:155-183 in the lazily normalised form):
// Hessenberg column from the dots and ||u_{j+1}||, the previous rotations, a new one, the residual
// estimate, the stop tests.
__global__ void k_barnoldi(BState S, BParams p, BKry K, int j) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.I || !S.lin_act[t]) return;
    const int m = S.m;
    double* hc = K.hcol + (long long)t * K.m1;
    double* sig = K.sig + (long long)t * K.m1;
    double* sig2 = K.sig2 + (long long)t * K.m1;
    double* H = S.H + (long long)t * (m + 1) * m;
    double* cs = S.cs + (long long)t * m;
    double* sn = S.sn + (long long)t * m;
    double* g = S.g + (long long)t * (m + 1);
    const double t2 = hc[j + 1];  // ||u_{j+1}||^2
    const double nrm = __dsqrt_rn(t2);
    sig2[j + 1] = t2 > 0.0 ? 1.0 / t2 : 0.0;
    sig[j + 1] = nrm > 0.0 ? 1.0 / nrm : 0.0;
    for (int i = 0; i <= j; ++i) H[i * m + j] = sig[j] * sig[i] * hc[i];
    H[(j + 1) * m + j] = nrm;  // the FP32 u_{j+1} carries sigma_j
    for (int i = 0; i < j; ++i) {
        const double a = cs[i] * H[i * m + j] + sn[i] * H[(i + 1) * m + j];
        H[(i + 1) * m + j] = -sn[i] * H[i * m + j] + cs[i] * H[(i + 1) * m + j];
        H[i * m + j] = a;
    }
    S.lmv[t] += 1;
    S.lpc[t] += 1;
    const double den = hypot(H[j * m + j], H[(j + 1) * m + j]);
    if (!(den > 0.0) || !isfinite(den)) {
        S.brk[t] = 1;
        S.lin_act[t] = 0;
        return;
    }
    cs[j] = H[j * m + j] / den;
    sn[j] = H[(j + 1) * m + j] / den;
    H[j * m + j] = den;
    H[(j + 1) * m + j] = 0.0;
    g[j + 1] = -sn[j] * g[j];
    g[j] = cs[j] * g[j];
    S.lit[t] += 1;
    K.kdone[t] = j + 1;
    const double rel = fabs(g[j + 1]) / S.bnorm[t];
    if (rel <= S.eta[t]) {
        S.lin_conv[t] = 1;
        S.lin_act[t] = 0;
    } else if (j + 1 >= m || S.lit[t] >= p.max_iters) {
        S.lin_act[t] = 0;  // the cycle is full (or the iteration budget spent): solution update, maybe restart
    } else {
        atomicOr(S.flags, kFlagLin);
    }
}

// End of a cycle: y from the triangular system (gmres.hpp:185-196), the update coefficients
// y_j sigma_j scaled to |c| <= 1 (the FP32 basis' double-FP32 combination), cmb = 1 for the update.
__global__ void k_bcycle_end(BState S, BKry K) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.I) return;
    S.cmb[t] = 0;
    if (!S.in_cyc[t] || S.brk[t]) return;
    const int m = S.m, k = K.kdone[t];
    const double* H = S.H + (long long)t * (m + 1) * m;
    const double* g = S.g + (long long)t * (m + 1);
    const double* sig = K.sig + (long long)t * K.m1;
    double* y = S.y + (long long)t * m;
    double* cf = K.coef + (long long)t * K.m;
    for (int ii = k - 1; ii >= 0; --ii) {
        const double piv = H[ii * m + ii];
        if (!(fabs(piv) > 0.0) || !isfinite(piv)) {
            S.brk[t] = 1;
            return;
        }
        double a = g[ii];
        for (int jj = ii + 1; jj < k; ++jj) a -= H[ii * m + jj] * y[jj];
        y[ii] = a / piv;
    }
    double scale = 0.0;
    for (int jj = 0; jj < k; ++jj) {
        cf[jj] = y[jj] * sig[jj];
        scale = fmax(scale, fabs(cf[jj]));
    }
    if (scale > 0.0)
        for (int jj = 0; jj < k; ++jj) cf[jj] /= scale;
    K.scale[t] = scale;
    S.cmb[t] = 1;
}

// After the solution update: a converged (or exhausted, or broken-down) linear solve ends and its
// counts go to the Newton counters (krylov_newton.hpp:88-93); otherwise the cycle restarts.
__device__ void bfinish_lin(BState& S, int t) {
    S.nJVP[t] += S.lmv[t];
    S.nlin[t] += S.lit[t];
    S.nprec[t] += S.lpc[t];
    if (!S.lin_conv[t]) S.nlinfail[t] += 1;
    S.in_cyc[t] = 0;
    if (S.brk[t]) S.nl_act[t] = 0;  // the reference leaves the Newton loop on a breakdown
}

__global__ void k_bafter_cycle(BState S, BParams p) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.I || !S.in_cyc[t]) return;
    S.assign[t] = 0;
    if (S.brk[t] || S.lin_conv[t] || S.lit[t] >= p.max_iters) {
        bfinish_lin(S, t);
        return;
    }
    S.rs_act[t] = 1;
    atomicOr(S.flags, kFlagRestart);
}

// A restart: beta = ||F - J z|| decides between convergence and a new cycle from u_0 = RN32(r / beta).
__global__ void k_brestart(BState S, BKry K) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.I || !S.rs_act[t]) return;
    S.lmv[t] += 1;
    const double beta = __dsqrt_rn(S.beta2[t]);
    if (beta / S.bnorm[t] <= S.eta[t]) {
        S.lin_conv[t] = 1;
        S.rs_act[t] = 0;
        bfinish_lin(S, t);
        return;
    }
    S.inv_beta[t] = 1.0 / beta;
    double* g = S.g + (long long)t * (S.m + 1);
    g[0] = beta;
    for (int i = 1; i <= S.m; ++i) g[i] = 0.0;
    K.sig[(long long)t * K.m1] = 1.0;
    K.sig2[(long long)t * K.m1] = 1.0;
    K.kdone[t] = 0;
    S.lin_act[t] = 1;
    atomicOr(S.flags, kFlagLin);
}

__global__ void k_bclear(int* a, int I) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < I) a[t] = 0;
}

// The line search of every instance whose linear solve ended (krylov_newton.hpp:95-104): the
// full step x - z was written by the solution update.
__global__ void k_bls_begin(BState S) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.I || !S.nl_act[t]) return;
    S.alpha[t] = 1.0;
    S.ls_act[t] = 1;
    S.eval[t] = 1;
    atomicOr(S.flags, kFlagLS);
}

// Armijo test of the trial just evaluated; on acceptance the trial becomes the iterate (the
// iterate buffers swap roles through cur), else the step halves, down to min_lambda.
__global__ void k_bls_test(BState S, BParams p) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.I || !S.ls_act[t]) return;
    const double fn = __dsqrt_rn(S.fn2[t]);
    S.nF[t] += 1;
    const double al = S.alpha[t];
    if (fn <= (1.0 - p.armijo * al) * S.rnorm[t]) {
        S.cur[t] ^= 1;
        S.rprev[t] = S.rnorm[t];
        S.rnorm[t] = fn;
        S.eta_prev[t] = S.eta[t];
        S.iters[t] += 1;
        S.ls_act[t] = 0;
        S.eval[t] = 0;
        return;
    }
    const double next = al * 0.5;
    S.alpha[t] = next;
    if (!(next >= p.min_lambda)) {
        S.ls_act[t] = 0;
        S.eval[t] = 0;
        S.nl_act[t] = 0;  // no acceptable step: the reference leaves the Newton loop
        return;
    }
    atomicOr(S.flags, kFlagLS);
}

__global__ void k_bfinal(BState S, BParams p) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.I) return;
    if (S.rnorm[t] <= p.rtol_nl * S.res0[t]) S.conv[t] = 1;
}

unsigned blocks_for(int I, int threads) { return (unsigned)((I + threads - 1) / threads); }

}  // namespace

// ------------------------------------------------------------------------------ the solver
struct BatchSolver::Impl {
    Context& ctx;
    KrylovParams kp;
    int I = 0, m = 0, pre = 2, post = 2;
    std::vector<int> n_of;          // per instance (table order)
    std::vector<double> lam_of;
    std::vector<long long> off_of;  // packed offsets
    std::vector<int> user_of;       // table order -> caller's index
    long long T = 0;
    BatchTuning tune;

    struct Cls {
        int n, t0, count;
        long long off0, N;
    };
    std::vector<Cls> cls;
    struct Pool {
        int s = 0, K = 0, top0 = 0, cls = -1;  // cls: the class whose finest level is s (-1: none)
        long long N = 0, pad = 0;
        DeviceArray<float> x, b, bs, r;
        DeviceArray<int> inst;
        MgPool view() const {
            return MgPool{x.p + pad, b.p, bs.p, r.p, N + 2 * pad, N + 64, N, inst.p};
        }
    };
    std::vector<std::unique_ptr<Pool>> pools;  // sizes n_max ... 15 (the last one is the tail)
    size_t tail_smem = 0;
    // Jacobian-aware tail (kp.coarse_jacobian): the coefficient c = lambda e^u of each pool grid below the
    // finest pool (natural layout, grid q at q s^3), and of the tail's levels 7, 3, 1 (grid q of the last pool)
    bool jac_tail = false;
    double tight = 0.0;  // forcing terms below this take the accurate product (kp.jvp_tight), else 0
    std::vector<DeviceArray<float>> cpool;
    DeviceArray<float> ctail[3];

    // packed vectors
    DeviceArray<double> xa, xb, F, z, R;
    // the exp table scaled by each instance's lambda (k_blam_tables)
    DeviceArray<double2> lt2;
    DeviceArray<float2> ltf;
    DeviceArray<float> c32, V32, Z32, W32, S32;
    // per-instance state
    DeviceArray<int> ibuf;
    DeviceArray<double> dbuf;
    DeviceArray<double> lam_d;
    BState S{};
    BKry K{};
    BParams bp{};
    // block table and partials
    DeviceArray<int> blk_inst, eb0, ebn, sb0, sbn;
    DeviceArray<long long> blk_beg, blk_end;
    int nblocks = 0;
    DeviceArray<double> partials;
    std::vector<BClass> ccfg;  // per class stencil shape (eval and J v)
    int* flags_h = nullptr;

    // captured graphs: one per Arnoldi step index, and the line-search trial
    std::vector<cudaGraphExec_t> step_graph;
    cudaGraphExec_t trial_graph = nullptr;

    Impl(Context& c) : ctx(c) {}
    ~Impl() {
        for (auto g : step_graph)
            if (g) cudaGraphExecDestroy(g);
        if (trial_graph) cudaGraphExecDestroy(trial_graph);
        if (flags_h) {
            std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
            cudaFreeHost(flags_h);
        }
    }

    void build_tables();
    void alloc_state();
    void vcycle(int j);
    void step(int j);
    void eval_all(int which);
    void trial();
    void restart();
    void combine(int kmax);
    int read_flags();
    void run_graph(cudaGraphExec_t& g, const std::function<void()>& body);
    void solve(double* x_out, numa_batch_result* res, double* seconds);
    void launch_dots(int cnt_total, const float* w);
    void launch_update(int j);
    void restrict_coef();
};

namespace {

bool batch_size_ok(size_t n) {
    // 2^k - 1 with k >= 5: odd down to the tail at 15 and an FP32 output on the finest level
    if (n < 31 || n > 1023) return false;
    return ((n + 1) & n) == 0;
}

}  // namespace

BatchSolver::BatchSolver(Context& ctx, const numa_batch_instance* inst, size_t count, const KrylovParams& p)
    : impl_(std::make_unique<Impl>(ctx)) {
    Impl& M = *impl_;
    if (count == 0) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "batched solver: no instances");
    if (p.restart == 0 || p.restart > kMaxRestart)
        throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "batched solver: restart length must be 1 .. 250");
    for (size_t i = 0; i < count; ++i)
        if (!batch_size_ok(inst[i].n))
            throw Status(NUMA_GPU_ERR_NOT_SUPPORTED,
                         "batched solver: grid sizes must be 2^k - 1 between 31 and 1023 (the FP32 multigrid "
                         "hierarchy ends in the one-CTA tail at 15)");
    M.kp = p;
    M.I = (int)count;
    M.m = (int)p.restart;
    M.jac_tail = p.coarse_jacobian;
    M.tight = p.jvp_tight ? 1e-5 : 0.0;
    // table order: larger grids first, then the caller's order
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [inst](int a, int b) { return inst[a].n > inst[b].n; });
    for (int t = 0; t < M.I; ++t) {
        const int u = order[t];
        M.user_of.push_back(u);
        M.n_of.push_back((int)inst[u].n);
        M.lam_of.push_back(inst[u].lambda);
        M.off_of.push_back(M.T);
        M.T += (long long)inst[u].n * inst[u].n * inst[u].n;
        if (M.cls.empty() || M.cls.back().n != (int)inst[u].n)
            M.cls.push_back(Impl::Cls{(int)inst[u].n, t, 0, M.off_of.back(),
                                      (long long)(inst[u].n * inst[u].n * inst[u].n)});
        M.cls.back().count += 1;
    }
    M.tune = BatchTuning{};
    M.alloc_state();
    M.build_tables();
}

BatchSolver::~BatchSolver() = default;

void BatchSolver::Impl::alloc_state() {
    const long long Tn = T;
    xa.resize(Tn);
    xb.resize(Tn);
    F.resize(Tn);
    z.resize(Tn);
    R.resize(Tn);
    c32.resize(Tn);
    W32.resize(Tn);
    S32.resize(Tn);
    V32.resize((size_t)(m + 1) * Tn);
    Z32.resize((size_t)m * Tn);
    // per-instance arrays
    const int ni = 22;
    ibuf.resize((size_t)ni * I + 8);
    int* ip = ibuf.p;
    int** iptrs[] = {&S.nl_act, &S.cur, &S.lin_act, &S.ls_act, &S.rs_act, &S.in_cyc, &S.assign, &S.lin_conv, &S.brk,
                     &S.eval, &S.cmb, &S.conv, &S.iters, &S.nF, &S.nJVP, &S.nlin, &S.nlinfail, &S.nprec, &S.lit,
                     &S.lmv, &S.lpc, &K.kdone};
    for (int q = 0; q < ni; ++q) *iptrs[q] = ip + (size_t)q * I;
    S.flags = ip + (size_t)ni * I;
    const int nd = 10;
    const size_t per = (size_t)nd + (m + 1) * m + 3 * m + 2 * (m + 1) + 3 * (m + 1) + m + 1;
    dbuf.resize(per * I);
    double* dp = dbuf.p;
    double** dptrs[] = {&S.res0, &S.rnorm, &S.rprev, &S.eta_prev, &S.eta, &S.alpha, &S.bnorm, &S.fn2, &S.beta2,
                        &S.inv_beta};
    for (int q = 0; q < nd; ++q) *dptrs[q] = dp + (size_t)q * I;
    double* q = dp + (size_t)nd * I;
    S.H = q;
    q += (size_t)(m + 1) * m * I;
    S.cs = q;
    q += (size_t)m * I;
    S.sn = q;
    q += (size_t)m * I;
    S.y = q;
    q += (size_t)m * I;
    S.g = q;
    q += (size_t)(m + 1) * I;
    K.hcol = q;
    q += (size_t)(m + 1) * I;
    K.sig = q;
    q += (size_t)(m + 1) * I;
    K.sig2 = q;
    q += (size_t)(m + 1) * I;
    K.coef = q;
    q += (size_t)m * I;
    K.scale = q;
    K.m1 = m + 1;
    K.m = m;
    S.I = I;
    S.m = m;
    lam_d.resize(I);
    NUMA_CUDA(cudaMemcpyAsync(lam_d.p, lam_of.data(), I * sizeof(double), cudaMemcpyHostToDevice, ctx.stream));
    lt2.resize((size_t)I << kExpTableBits);
    ltf.resize((size_t)I << kExpTableBits);
    for (int t0 = 0; t0 < I; t0 += 65535) {
        k_blam_tables<<<dim3((1 << kExpTableBits) / 256, std::min(65535, I - t0)), 256, 0, ctx.stream>>>(lam_d.p, lt2.p,
                                                                                                      ltf.p, t0);
        ctx.count_launch();
    }
    ctx.check_launch("batched lambda tables");
    bp = BParams{kp.rtol_nl, kp.eta_init, kp.eta_max, kp.gamma, kp.alpha, kp.armijo, kp.min_lambda,
                 (int)std::min<size_t>(kp.max_iters, (size_t)1 << 30)};
    {
        std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
        NUMA_CUDA(cudaMallocHost(reinterpret_cast<void**>(&flags_h), sizeof(int)));
    }
    // multigrid pools: sizes n_max, (n_max - 1) / 2, ..., 15
    std::vector<int> top_of_size;
    for (int s = cls.front().n; s >= 15; s = (s - 1) / 2) {
        auto P = std::make_unique<Pool>();
        P->s = s;
        P->N = (long long)s * s * s;
        P->pad = ((long long)(s * s - 1) / 2 + s + 2 + 31) / 32 * 32;
        std::vector<int> insts;
        for (int t = 0; t < I; ++t)
            if (n_of[t] >= s) insts.push_back(t);
        P->K = (int)insts.size();
        P->top0 = P->K;
        for (int c = 0; c < (int)cls.size(); ++c)
            if (cls[c].n == s) {
                P->cls = c;
                P->top0 = P->K - cls[c].count;
            }
        P->x.resize((size_t)P->K * (P->N + 2 * P->pad));
        P->b.resize((size_t)P->K * (P->N + 64));
        P->bs.resize((size_t)P->K * (P->N + 64));
        if (s > 15) P->r.resize((size_t)P->K * P->N);
        P->inst.resize(P->K);
        NUMA_CUDA(cudaMemcpyAsync(P->inst.p, insts.data(), P->K * sizeof(int), cudaMemcpyHostToDevice, ctx.stream));
        // padding and untouched halves read by the unconditional loads must be finite
        NUMA_CUDA(cudaMemsetAsync(P->x.p, 0, P->x.n * sizeof(float), ctx.stream));
        NUMA_CUDA(cudaMemsetAsync(P->b.p, 0, P->b.n * sizeof(float), ctx.stream));
        NUMA_CUDA(cudaMemsetAsync(P->bs.p, 0, P->bs.n * sizeof(float), ctx.stream));
        pools.push_back(std::move(P));
    }
    if (jac_tail) {
        cpool.resize(pools.size());
        for (size_t q = 1; q < pools.size(); ++q) cpool[q].resize((size_t)pools[q]->K * pools[q]->N);
        const int Kt = pools.back()->K;
        ctail[0].resize((size_t)Kt * 343);
        ctail[1].resize((size_t)Kt * 27);
        ctail[2].resize((size_t)Kt);
    }
    // the tail: levels 15, 7, 3, 1 of every instance in one CTA each (and, Jacobian-aware, c h^2 of each)
    size_t elems = 0;
    for (int s = 15; s >= 1; s = (s - 1) / 2) {
        elems += (jac_tail ? 4 : 3) * (size_t)s * s * s;
        if (s == 1) break;
    }
    elems += 15 * 15 * 15;
    tail_smem = elems * sizeof(float);
    const int lim = set_dynamic_smem_limit(ctx, k_btail);
    if (tail_smem > (size_t)lim) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "batched multigrid tail exceeds shared memory");
    ctx.sync();
}

void BatchSolver::Impl::build_tables() {
    // element-wise block table
    const long long E = std::max(1024, tune.elems_per_block);
    std::vector<int> bi, b0(I), bn(I);
    std::vector<long long> bb, be;
    for (int t = 0; t < I; ++t) {
        const long long N = (long long)n_of[t] * n_of[t] * n_of[t];
        b0[t] = (int)bi.size();
        for (long long s = 0; s < N; s += E) {
            bi.push_back(t);
            bb.push_back(off_of[t] + s);
            be.push_back(off_of[t] + std::min(N, s + E));
        }
        bn[t] = (int)bi.size() - b0[t];
    }
    nblocks = (int)bi.size();
    blk_inst.resize(nblocks);
    blk_beg.resize(nblocks);
    blk_end.resize(nblocks);
    eb0.resize(I);
    ebn.resize(I);
    NUMA_CUDA(cudaMemcpyAsync(blk_inst.p, bi.data(), nblocks * sizeof(int), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(blk_beg.p, bb.data(), nblocks * sizeof(long long), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(blk_end.p, be.data(), nblocks * sizeof(long long), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(eb0.p, b0.data(), I * sizeof(int), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(ebn.p, bn.data(), I * sizeof(int), cudaMemcpyHostToDevice, ctx.stream));
    // stencil shapes and their partial slots (the residual's norm)
    ccfg.clear();
    std::vector<int> s0(I), sn(I);
    int slots = 0;
    for (const Cls& c : cls) {
        BClass b{};
        b.n = c.n;
        b.t0 = c.t0;
        b.kb = (c.n + kBX - 1) / kBX;
        b.jb = (c.n + kBY - 1) / kBY;
        b.ichunk = std::max(1, std::min(c.n, tune.planes));
        b.zch = (c.n + b.ichunk - 1) / b.ichunk;
        b.N = c.N;
        b.off0 = c.off0;
        b.h2inv = ((double)c.n + 1.0) * ((double)c.n + 1.0);
        b.h2inv32 = (float)b.h2inv;
        b.pbase = slots;
        const int per = b.kb * b.jb * b.zch;
        for (int g = 0; g < c.count; ++g) {
            s0[c.t0 + g] = slots + g * per;
            sn[c.t0 + g] = per;
        }
        slots += per * c.count;
        ccfg.push_back(b);
    }
    sb0.resize(I);
    sbn.resize(I);
    NUMA_CUDA(cudaMemcpyAsync(sb0.p, s0.data(), I * sizeof(int), cudaMemcpyHostToDevice, ctx.stream));
    NUMA_CUDA(cudaMemcpyAsync(sbn.p, sn.data(), I * sizeof(int), cudaMemcpyHostToDevice, ctx.stream));
    partials.resize(std::max<size_t>((size_t)nblocks * kCgsBlock, (size_t)slots) + 64);
    // graphs captured with the old tables are stale
    for (auto& g : step_graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    step_graph.assign(m, nullptr);
    if (trial_graph) {
        cudaGraphExecDestroy(trial_graph);
        trial_graph = nullptr;
    }
    ctx.sync();
}

// Launches a stencil kernel over one class in chunks of grids that keep gridDim.z <= 65535.
template <class Launch>
static void over_class(const BClass& c, int count, Launch&& launch) {
    const int per = std::max(1, 65535 / c.zch);
    for (int g0 = 0; g0 < count; g0 += per) {
        BClass cc = c;
        const int cnt = std::min(per, count - g0);
        cc.t0 = c.t0 + g0;
        cc.off0 = c.off0 + (long long)g0 * c.N;
        cc.pbase = c.pbase + g0 * c.kb * c.jb * c.zch;
        launch(cc, dim3(c.kb, c.jb, cnt * c.zch));
    }
}

// Launches a pool kernel over grids [g0, g0 + count) in chunks with count * zch <= 65535 blocks in z.
template <class Launch>
static void over_pool(int g0, int count, int zch, Launch&& launch) {
    const int per = std::max(1, 65535 / zch);
    for (int a = g0; a < g0 + count; a += per) launch(a, std::min(per, g0 + count - a));
}

void BatchSolver::Impl::vcycle(int j) {
    cudaStream_t s = ctx.stream;
    const dim3 blk(BX, BY);
    const int* act = S.lin_act;
    const int np = (int)pools.size();
    const float* u = V32.p + (size_t)j * T;
    float* zout = Z32.p + (size_t)j * T;
    auto pass = [&](Pool& P, int g0, int count, int mode, int c, float* z32, long long zs) {
        const Split g = make_split(P.s);
        const MgPool V = P.view();
        const int n = P.s;
        const int zch = n >= 64 ? (n + 3) / 4 : n;
        const dim3 grid0(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, 1);
        over_pool(g0, count, zch, [&](int a, int cnt) {
            const dim3 grid(grid0.x, grid0.y, cnt * zch);
            float* zq = z32 ? z32 + (long long)(a - g0) * zs : nullptr;
            if (mode == kPassLastZ) {
                if (n >= 64) launch_pdl(k_bpass<kPassLastZ, 4, 0>, grid, blk, 0, s, V, act, a, zch, g, c, zq, zs);
                else launch_pdl(k_bpass<kPassLastZ, 1, 0>, grid, blk, 0, s, V, act, a, zch, g, c, zq, zs);
            } else {
                if (n == 127) launch_pdl(k_bpass<kPassFull, 4, 127>, grid, blk, 0, s, V, act, a, zch, g, c, zq, zs);
                else if (n == 255) launch_pdl(k_bpass<kPassFull, 4, 255>, grid, blk, 0, s, V, act, a, zch, g, c, zq, zs);
                else if (n >= 64) launch_pdl(k_bpass<kPassFull, 4, 0>, grid, blk, 0, s, V, act, a, zch, g, c, zq, zs);
                else launch_pdl(k_bpass<kPassFull, 1, 0>, grid, blk, 0, s, V, act, a, zch, g, c, zq, zs);
            }
            ctx.count_launch();
        });
    };
    // down: right-hand sides, pre-smoothing, residual, restriction
    for (int p = 0; p + 1 < np; ++p) {
        Pool& P = *pools[p];
        const int n = P.s;
        const Split g = make_split(n);
        const MgPool V = P.view();
        if (P.cls >= 0) {
            const Cls& c = cls[P.cls];
            const int blocks = (int)std::min<long long>((g.half + 255) / 256, (long long)ctx.sm_count * 4);
            const float inv = (float)(1.0 / (((double)n + 1.0) * ((double)n + 1.0)));
            for (int a = 0; a < c.count; a += 65535) {
                const int cnt = std::min(65535, c.count - a);
                launch_pdl(k_bscale_in<true>, dim3(blocks, cnt), 256, 0, s, u + c.off0 + (long long)a * c.N, c.N, V, act,
                           P.top0 + a, inv, (int)P.N, g.half);
                ctx.count_launch();
            }
        }
        // pre-smoothing: the first colour-0 pass came with the right-hand side
        for (int sw = 0; sw < pre; ++sw) {
            if (sw > 0) pass(P, 0, P.K, kPassFull, 0, nullptr, 0);
            pass(P, 0, P.K, kPassFull, 1, nullptr, 0);
        }
        {
            const int zch = (n + 1) / 2;
            const dim3 g0(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, 1);
            over_pool(0, P.K, zch, [&](int a, int cnt) {
                MgPool W = V;
                W.x += (long long)a * V.sx;
                W.b += (long long)a * V.sb;
                W.r += (long long)a * V.sr;
                W.inst += a;
                launch_pdl(k_bresidual, dim3(g0.x, g0.y, cnt * zch), blk, 0, s, W, act, zch, g,
                           (float)(((double)n + 1.0) * ((double)n + 1.0)));
                ctx.count_launch();
            });
        }
        Pool& C = *pools[p + 1];
        const int nc = C.s;
        const Split gc = make_split(nc);
        const bool fused = (p + 2 < np);  // the tail level's first pass is its own
        const MgPool CV = C.view();
        const int zc = (nc + 1) / 2;  // two coarse planes a thread
        over_pool(0, P.K, zc, [&](int a, int cnt) {
            MgPool Fw = V, Cw = CV;
            Fw.r += (long long)a * V.sr;
            Fw.inst += a;
            Cw.x += (long long)a * CV.sx;
            Cw.b += (long long)a * CV.sb;
            Cw.bs += (long long)a * CV.sb;
            Cw.inst += a;
            const dim3 rg((nc + BX - 1) / BX, (nc + BY - 1) / BY, cnt * zc);
            const float invc = (float)(1.0 / (((double)nc + 1.0) * ((double)nc + 1.0)));
            if (fused) launch_pdl(k_brestrict<true>, rg, blk, 0, s, Fw, Cw, act, n, nc, gc.half, invc);
            else launch_pdl(k_brestrict<false>, rg, blk, 0, s, Fw, Cw, act, n, nc, gc.half, invc);
            ctx.count_launch();
        });
    }
    // the tail of every grid
    {
        Pool& P = *pools[np - 1];
        TailParams tp{};
        int l = 0;
        for (int sz = 15; l < kMaxTail; sz = (sz - 1) / 2) {
            const double h2 = ((double)sz + 1.0) * ((double)sz + 1.0);
            tp.n[l] = sz;
            tp.h2inv[l] = h2;
            tp.inv[l] = 1.0 / h2;
            tp.six_h2inv[l] = 6.0 * h2;
            ++l;
            if (sz == 1) break;
        }
        tp.levels = l;
        tp.pre = pre;
        tp.post = post;
        tp.half = make_split(15).half;
        for (int m2 = 0; m2 < kMaxTail; ++m2) tp.c[m2] = nullptr;
        const MgPool V = P.view();
        for (int a = 0; a < P.K; a += 65535) {
            MgPool W = V;
            W.x += (long long)a * V.sx;
            W.b += (long long)a * V.sb;
            W.bs += (long long)a * V.sb;
            W.inst += a;
            TailParams ta = tp;
            if (jac_tail) {  // levels 15, 7, 3, 1 of grid a onwards
                ta.c[0] = cpool[np - 1].p + (size_t)a * 3375;
                ta.c[1] = ctail[0].p + (size_t)a * 343;
                ta.c[2] = ctail[1].p + (size_t)a * 27;
                ta.c[3] = ctail[2].p + (size_t)a;
            }
            launch_pdl(k_btail, std::min(65535, P.K - a), 1024, tail_smem, s, W, act, ta);
            ctx.count_launch();
        }
    }
    // up: prolongation and post-smoothing; the finest level of each instance writes z_j
    for (int p = np - 2; p >= 0; --p) {
        Pool& P = *pools[p];
        Pool& C = *pools[p + 1];
        const int n = P.s, nc = C.s;
        const Split g = make_split(n), gc = make_split(nc);
        const MgPool V = P.view(), CV = C.view();
        over_pool(0, P.K, nc + 1, [&](int a, int cnt) {
            MgPool Fw = V, Cw = CV;
            Fw.x += (long long)a * V.sx;
            Fw.inst += a;
            Cw.x += (long long)a * CV.sx;
            Cw.inst += a;
            const dim3 cg((nc + 1 + BX - 1) / BX, (nc + 1 + BY - 1) / BY, cnt * (nc + 1));
            launch_pdl(k_bprolong<false>, cg, blk, 0, s, Cw, Fw, act, nc, gc.half, n, g.half);
            ctx.count_launch();
        });
        for (int sw = 0; sw < post; ++sw) {
            pass(P, 0, P.K, kPassFull, 1, nullptr, 0);
            const bool last = sw + 1 == post;
            if (!last || P.cls < 0) {
                pass(P, 0, P.K, kPassFull, 0, nullptr, 0);
            } else {
                if (P.top0 > 0) pass(P, 0, P.top0, kPassFull, 0, nullptr, 0);
                const Cls& c = cls[P.cls];
                pass(P, P.top0, c.count, kPassLastZ, 0, zout + c.off0, c.N);
            }
        }
    }
}

// h_r = <w, u_r> for r <= j (blocks of kCgsBlock vectors), reduced per instance into hcol
void BatchSolver::Impl::launch_dots(int cnt_total, const float* w) {
    cudaStream_t s = ctx.stream;
    const BlkTab B{blk_inst.p, blk_beg.p, blk_end.p};
    for (int b0 = 0; b0 < cnt_total; b0 += kCgsBlock) {
        const int c = std::min(kCgsBlock, cnt_total - b0);
        switch (c) {
#define NUMA_BDOTS(KK)                                                                                         \
    case KK:                                                                                                   \
        launch_pdl(k_bdots<KK>, nblocks, kEwThreads, 0, s, w, (const float*)V32.p, T, b0, B, (const int*)S.lin_act, \
                   partials.p);                                                                                \
        break;
            NUMA_BDOTS(1) NUMA_BDOTS(2) NUMA_BDOTS(3) NUMA_BDOTS(4) NUMA_BDOTS(5) NUMA_BDOTS(6) NUMA_BDOTS(7) NUMA_BDOTS(8)
#undef NUMA_BDOTS
        }
        launch_pdl(k_bsegsum, (unsigned)((I + 3) / 4), 128, 0, s, (const double*)partials.p, c, (const int*)eb0.p,
                   (const int*)ebn.p, (const int*)S.lin_act, I, K.hcol, K.m1, b0);
        ctx.count_launch(2);
    }
}

// u_{j+1} = RN32(sigma_j (w - sum h_r sigma_r^2 u_r)) and ||u_{j+1}||^2 into hcol[j + 1]
void BatchSolver::Impl::launch_update(int j) {
    cudaStream_t s = ctx.stream;
    const BlkTab B{blk_inst.p, blk_beg.p, blk_end.p};
    const int cnt = j + 1;
    // the double-FP32 partial sums of a basis longer than one block: T float2 in the FP64 scratch R
    float2* part = reinterpret_cast<float2*>(R.p);
    for (int b0 = 0; b0 < cnt; b0 += kCgsBlock) {
        const int c = std::min(kCgsBlock, cnt - b0);
        const bool last = b0 + c >= cnt, first = b0 == 0;
        switch (c) {
#define NUMA_BUPD(KK)                                                                                          \
    case KK:                                                                                                   \
        if (last)                                                                                              \
            launch_pdl(k_bupdate<KK, true>, nblocks, kEwThreads, 0, s, (const float*)W32.p, part, V32.p, T, j, b0, \
                       first, B, (const int*)S.lin_act, K, partials.p);                                        \
        else                                                                                                   \
            launch_pdl(k_bupdate<KK, false>, nblocks, kEwThreads, 0, s, (const float*)W32.p, part, V32.p, T, j, b0, \
                       first, B, (const int*)S.lin_act, K, partials.p);                                        \
        break;
            NUMA_BUPD(1) NUMA_BUPD(2) NUMA_BUPD(3) NUMA_BUPD(4) NUMA_BUPD(5) NUMA_BUPD(6) NUMA_BUPD(7) NUMA_BUPD(8)
#undef NUMA_BUPD
        }
        ctx.count_launch();
    }
    launch_pdl(k_bsegsum, (unsigned)((I + 3) / 4), 128, 0, s, (const double*)partials.p, 1, (const int*)eb0.p,
               (const int*)ebn.p, (const int*)S.lin_act, I, K.hcol, K.m1, j + 1);
    ctx.count_launch();
}

// The Jacobian coefficient of every pool level below each instance's finest and of the tail levels,
// restricted from RN32(lambda e^u) of the current iterates (k_beval's c32), for the instances still in
// Newton: the single-instance Jacobian-aware hierarchy's restriction chain (PoissonMG::set_coarse_coefficient).
void BatchSolver::Impl::restrict_coef() {
    cudaStream_t s = ctx.stream;
    const dim3 blk(BX, BY);
    const int np = (int)pools.size();
    auto launch = [&](const float* src, long long ss, float* dst, long long sd, const int* inst, int g0, int count,
                      int nf, int nc) {
        const int ichunk = nc >= 64 ? 8 : (nc >= 16 ? 4 : 1);
        const int zch = (nc + ichunk - 1) / ichunk;
        over_pool(0, count, zch, [&](int a, int cnt) {
            const dim3 grid((nc + BX - 1) / BX, (nc + BY - 1) / BY, cnt * zch);
            launch_pdl(k_brestrict_coef, grid, blk, 0, s, src + (long long)a * ss, ss, dst, sd, inst,
                       (const int*)S.nl_act, g0 + a, nf, nc, ichunk, zch);
            ctx.count_launch();
        });
    };
    for (int p = 1; p < np; ++p) {
        Pool& F = *pools[p - 1];
        Pool& C = *pools[p];
        const int nf = F.s, nc = C.s;
        // grids whose finest level is finer than nf: from the finer pool's coefficients
        if (p >= 2 && F.top0 > 0)
            launch(cpool[p - 1].p, F.N, cpool[p].p, C.N, F.inst.p, 0, F.top0, nf, nc);
        // grids whose finest level is nf: from the class's RN32(lambda e^u)
        if (F.cls >= 0) {
            const Cls& c = cls[F.cls];
            launch(c32.p + c.off0, c.N, cpool[p].p, C.N, F.inst.p, F.top0, c.count, nf, nc);
        }
    }
    // the tail levels 7, 3, 1 from level 15 (every instance)
    const int Kt = pools.back()->K;
    launch(cpool[np - 1].p, 3375, ctail[0].p, 343, pools.back()->inst.p, 0, Kt, 15, 7);
    launch(ctail[0].p, 343, ctail[1].p, 27, pools.back()->inst.p, 0, Kt, 7, 3);
    launch(ctail[1].p, 27, ctail[2].p, 1, pools.back()->inst.p, 0, Kt, 3, 1);
    ctx.check_launch("batched coarse coefficients");
}

// One Arnoldi step j of every instance whose linear solve is active.
void BatchSolver::Impl::step(int j) {
    cudaStream_t s = ctx.stream;
    vcycle(j);
    const float* zj = Z32.p + (size_t)j * T;
    for (const BClass& c : ccfg) {
        const int count = cls[&c - ccfg.data()].count;
        over_class(c, count, [&](const BClass& cc, dim3 grid) {
            launch_pdl(k_bjvp32f, grid, dim3(kBX, kBY), 0, s, (const float*)c32.p, zj, W32.p, (const int*)S.lin_act, cc,
                       tight > 0.0 ? (const double*)S.eta : nullptr, tight);
            ctx.count_launch();
        });
    }
    launch_dots(j + 1, W32.p);
    launch_update(j);
    NUMA_CUDA(cudaMemsetAsync(S.flags, 0, sizeof(int), s));
    launch_pdl(k_barnoldi, blocks_for(I, kScalarThreads), kScalarThreads, 0, s, S, bp, K, j);
    ctx.count_launch();
}

// F, c32, RN32(F) (into u_0) and the residual norms of the instances marked in S.eval, at x[cur]
// (which = 0) or at the trial point x[1 - cur] (which = 1); ||F||^2 into S.fn2.
void BatchSolver::Impl::eval_all(int which) {
    cudaStream_t s = ctx.stream;
    for (size_t ci = 0; ci < ccfg.size(); ++ci) {
        const BClass& c = ccfg[ci];
        over_class(c, cls[ci].count, [&](const BClass& cc, dim3 grid) {
            launch_pdl(k_beval, grid, dim3(kBX, kBY), 0, s, (const double*)xa.p, (const double*)xb.p, (const int*)S.cur,
                       which, (const int*)S.eval, (const double*)lam_d.p, cc, F.p, c32.p, V32.p, partials.p,
                       (const double2*)lt2.p, (const float2*)ltf.p);
            ctx.count_launch();
        });
    }
    launch_pdl(k_bsegsum, (unsigned)((I + 3) / 4), 128, 0, s, (const double*)partials.p, 1, (const int*)sb0.p,
               (const int*)sbn.p, (const int*)S.eval, I, S.fn2, 1, 0);
    ctx.count_launch();
}

// One line-search trial of every instance still searching: F at its trial point, the Armijo
// test, and for the rejected ones the next, halved trial point.
void BatchSolver::Impl::trial() {
    cudaStream_t s = ctx.stream;
    eval_all(1);
    NUMA_CUDA(cudaMemsetAsync(S.flags, 0, sizeof(int), s));
    launch_pdl(k_bls_test, blocks_for(I, kScalarThreads), kScalarThreads, 0, s, S, bp);
    const BlkTab B{blk_inst.p, blk_beg.p, blk_end.p};
    launch_pdl(k_bstep, nblocks, kEwThreads, 0, s, (const double*)z.p, (const double*)xa.p, xb.p, (const int*)S.cur,
               (const int*)S.ls_act, (const double*)S.alpha, B);
    ctx.count_launch(2);
}

// The solution update of the cycle just finished (and the full step x - z), kmax the longest basis.
void BatchSolver::Impl::combine(int kmax) {
    cudaStream_t s = ctx.stream;
    launch_pdl(k_bcycle_end, blocks_for(I, kScalarThreads), kScalarThreads, 0, s, S, K);
    ctx.count_launch();
    const BlkTab B{blk_inst.p, blk_beg.p, blk_end.p};
    // blocks of kCgsBlock basis vectors: the first assigns (on a first cycle) or adds, the others add,
    // the last also writes the full step x - z
    const int kk = std::max(kmax, 1);
    for (int b0 = 0; b0 < kk; b0 += kCgsBlock) {
        const int c = std::min(kCgsBlock, kk - b0);
        const bool first = b0 == 0, last = b0 + c >= kk;
        switch (c) {
#define NUMA_BCMB(KK)                                                                                         \
    case KK:                                                                                                  \
        launch_pdl(k_bcombine<KK>, nblocks, kEwThreads, 0, s, (const float*)Z32.p, T, b0, first, last, z.p,    \
                   (const double*)xa.p, xb.p, (const int*)S.cur, (const int*)S.cmb, (const int*)S.assign, B, K); \
        break;
            NUMA_BCMB(1) NUMA_BCMB(2) NUMA_BCMB(3) NUMA_BCMB(4) NUMA_BCMB(5) NUMA_BCMB(6) NUMA_BCMB(7) NUMA_BCMB(8)
#undef NUMA_BCMB
        }
        ctx.count_launch();
    }
    NUMA_CUDA(cudaMemsetAsync(S.flags, 0, sizeof(int), s));
    launch_pdl(k_bafter_cycle, blocks_for(I, kScalarThreads), kScalarThreads, 0, s, S, bp);
    ctx.count_launch();
}

// Restart of the cycles that ended unconverged: r = F - J z, then either convergence or a new cycle.
void BatchSolver::Impl::restart() {
    cudaStream_t s = ctx.stream;
    const BlkTab B{blk_inst.p, blk_beg.p, blk_end.p};
    launch_pdl(k_bto32, nblocks, kEwThreads, 0, s, (const double*)z.p, S32.p, (const int*)S.rs_act, B);
    ctx.count_launch();
    for (size_t ci = 0; ci < ccfg.size(); ++ci)
        over_class(ccfg[ci], cls[ci].count, [&](const BClass& cc, dim3 grid) {
            launch_pdl(k_bjvp32f, grid, dim3(kBX, kBY), 0, s, (const float*)c32.p, (const float*)S32.p, W32.p,
                       (const int*)S.rs_act, cc, tight > 0.0 ? (const double*)S.eta : nullptr, tight);
            ctx.count_launch();
        });
    launch_pdl(k_bsub, nblocks, kEwThreads, 0, s, (const double*)F.p, (const float*)W32.p, R.p, (const int*)S.rs_act, B,
               partials.p);
    launch_pdl(k_bsegsum, (unsigned)((I + 3) / 4), 128, 0, s, (const double*)partials.p, 1, (const int*)eb0.p,
               (const int*)ebn.p, (const int*)S.rs_act, I, S.beta2, 1, 0);
    NUMA_CUDA(cudaMemsetAsync(S.flags, 0, sizeof(int), s));
    launch_pdl(k_brestart, blocks_for(I, kScalarThreads), kScalarThreads, 0, s, S, K);
    launch_pdl(k_bscale32, nblocks, kEwThreads, 0, s, (const double*)R.p, V32.p, (const double*)S.inv_beta,
               (const int*)S.lin_act, B);
    launch_pdl(k_bclear, blocks_for(I, kScalarThreads), kScalarThreads, 0, s, S.rs_act, I);
    ctx.count_launch(5);
}

int BatchSolver::Impl::read_flags() {
    NUMA_CUDA(cudaMemcpyAsync(flags_h, S.flags, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
    NUMA_CUDA(cudaStreamSynchronize(ctx.stream));
    return *flags_h;
}

// Replays body's kernels as a CUDA graph, capturing them on first use.
void BatchSolver::Impl::run_graph(cudaGraphExec_t& g, const std::function<void()>& body) {
    if (!g) {
        std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
        const uint64_t before = ctx.launches;
        NUMA_CUDA(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal));
        cudaGraph_t graph = nullptr;
        try {
            body();
        } catch (...) {
            cudaStreamEndCapture(ctx.stream, &graph);
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            throw;
        }
        NUMA_CUDA(cudaStreamEndCapture(ctx.stream, &graph));
        const cudaError_t e = cudaGraphInstantiate(&g, graph, 0);
        cudaGraphDestroy(graph);
        NUMA_CUDA(e);
        ctx.launches = before;
    }
    NUMA_CUDA(cudaGraphLaunch(g, ctx.stream));
}

void BatchSolver::Impl::solve(double* x_out, numa_batch_result* res, double* seconds) {
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = ctx.stream;
    const unsigned sb = blocks_for(I, kScalarThreads);
    NUMA_CUDA(cudaMemsetAsync(xa.p, 0, (size_t)T * sizeof(double), s));
    launch_pdl(k_binit, sb, kScalarThreads, 0, s, S);
    ctx.count_launch();
    eval_all(0);
    launch_pdl(k_bfirst, sb, kScalarThreads, 0, s, S, bp);
    ctx.count_launch();
    for (size_t k = 0; k < kp.max_nl; ++k) {
        NUMA_CUDA(cudaMemsetAsync(S.flags, 0, sizeof(int), s));
        launch_pdl(k_bnl_begin, sb, kScalarThreads, 0, s, S, bp, K, (int)k);
        ctx.count_launch();
        if (!(read_flags() & kFlagNL)) break;
        if (jac_tail) restrict_coef();  // the coarse levels' Jacobian at the new iterates
        // FGMRES: cycles of up to m steps, restarts while an instance needs one (every cycle adds at
        // least one iteration to each instance it runs, so gmres_max_iters bounds the cycles)
        for (size_t cycle = 0; cycle <= kp.max_iters; ++cycle) {
            int steps = 0;
            for (int j = 0; j < m; ++j) {
                run_graph(step_graph[j], [&] { step(j); });
                ++steps;
                if (!(read_flags() & kFlagLin)) break;
            }
            combine(steps);
            if (!(read_flags() & kFlagRestart)) break;
            restart();
            if (!(read_flags() & kFlagLin)) break;
        }
        // line search
        NUMA_CUDA(cudaMemsetAsync(S.flags, 0, sizeof(int), s));
        launch_pdl(k_bls_begin, sb, kScalarThreads, 0, s, S);
        ctx.count_launch();
        int guard = 0;
        while ((read_flags() & kFlagLS) && guard++ < 64) run_graph(trial_graph, [&] { trial(); });
    }
    launch_pdl(k_bfinal, sb, kScalarThreads, 0, s, S, bp);
    ctx.count_launch();
    ctx.check_launch("batched solve");
    // results
    std::vector<int> hi((size_t)22 * I);
    std::vector<double> hd((size_t)10 * I);
    NUMA_CUDA(cudaMemcpyAsync(hi.data(), ibuf.p, hi.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
    NUMA_CUDA(cudaMemcpyAsync(hd.data(), dbuf.p, hd.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    NUMA_CUDA(cudaStreamSynchronize(s));
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    auto iv = [&](int field, int t) { return hi[(size_t)field * I + t]; };
    auto dv = [&](int field, int t) { return hd[(size_t)field * I + t]; };
    for (int t = 0; t < I; ++t) {
        numa_batch_result& o = res[user_of[t]];
        o.converged = iv(11, t);
        o.status = 0;  // a breakdown or a failed line search ends the instance unconverged, as in the reference
        o.iters = (uint64_t)iv(12, t);
        o.n_F = (uint64_t)iv(13, t);
        o.n_JVP = (uint64_t)iv(14, t);
        o.n_lin_iters = (uint64_t)iv(15, t);
        o.n_prec = (uint64_t)iv(17, t);
        o.res_rel = dv(0, t) > 0.0 ? dv(1, t) / dv(0, t) : dv(1, t);
        o.seconds = secs;
    }
    if (x_out) {
        // the caller's packed host buffer, instances in the caller's order
        std::vector<long long> uoff(I + 1, 0);
        std::vector<long long> nn(I);
        for (int t = 0; t < I; ++t) nn[user_of[t]] = (long long)n_of[t] * n_of[t] * n_of[t];
        for (int u = 0; u < I; ++u) uoff[u + 1] = uoff[u] + nn[u];
        for (int t = 0; t < I; ++t) {
            const double* src = (iv(1, t) ? xb.p : xa.p) + off_of[t];
            NUMA_CUDA(cudaMemcpyAsync(x_out + uoff[user_of[t]], src, (size_t)nn[user_of[t]] * sizeof(double),
                                      cudaMemcpyDeviceToHost, s));
        }
        NUMA_CUDA(cudaStreamSynchronize(s));
    }
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void BatchSolver::solve(double* x_out, numa_batch_result* results, double* seconds) {
    impl_->solve(x_out, results, seconds);
}

size_t BatchSolver::instances() const { return (size_t)impl_->I; }
size_t BatchSolver::total_unknowns() const { return (size_t)impl_->T; }
BatchTuning BatchSolver::tuning() const { return impl_->tune; }

void BatchSolver::set_tuning(const BatchTuning& t) {
    BatchTuning c = t;
    c.planes = std::max(1, std::min(c.planes, 64));
    c.elems_per_block = std::max(1024, std::min(c.elems_per_block, 1 << 22));
    impl_->tune = c;
    impl_->build_tables();
}

// Times one batched solve for each candidate tile shape (planes a thread marches in the residual
// and Jacobian kernels, elements a block of the element-wise passes), after one warm solve, and
// keeps the fastest.
BatchTuning BatchSolver::autotune(const int* planes, int np, const int* elems, int ne, double* seconds) {
    BatchTuning best = impl_->tune;
    double best_t = -1.0;
    std::vector<numa_batch_result> r(impl_->I);
    int idx = 0;
    for (int a = 0; a < np; ++a)
        for (int b = 0; b < ne; ++b, ++idx) {
            BatchTuning c{};
            c.planes = planes[a];
            c.elems_per_block = elems[b];
            set_tuning(c);
            double t = 0.0;
            solve(nullptr, r.data(), &t);  // warm: graphs captured for these tables
            solve(nullptr, r.data(), &t);
            if (seconds) seconds[idx] = t;
            if (best_t < 0.0 || t < best_t) {
                best_t = t;
                best = impl_->tune;
            }
        }
    set_tuning(best);
    return best;
}

}  // namespace numa::gpu
