// poisson_mg.cu — geometric-multigrid V-cycle for -Laplacian_h (linalg/poisson_mg.hpp) on the GPU.
//
// Same hierarchy as the reference: levels while n is odd, (n-1)/2 and h^-2/4 per level, down to
// n = 1 (poisson_mg.hpp:44-63); red-black Gauss-Seidel with colour (i+j+k)&1, order 0 = colour
// 0 then 1 for pre-smoothing and order 1 for post-smoothing (:99-126, :278-293); 27-point full
// weighting (:152-188); trilinear additive prolongation (:191-260); coarsest level exact at
// n = 1, else 30 alternating sweeps (:266-275).
//
// GB300 choices (FP64 is the scarce resource, ~1.2 TFLOP/s; FP32 runs at HBM speed):
//  * b h^2 is formed once per level and cycle (the reference recomputes b*inv in every sweep:
//    the stored product is the same rounded value);
//  * x / 6 uses the 3-operation correctly rounded division (div6);
//  * the first pass of a level, whose x is zero, reads no neighbours (they are +0.0), and no
//    level's x is zero-filled: every value the reference would read as zero is overwritten
//    before it is read;
//  * prolongation is added only at colour-0 points when post-smoothing follows: the first
//    post-smoothing pass overwrites every colour-1 point without reading it;
//  * the finest level of the FP64 cycle smooths directly in the output vector z and reads r in
//    place, so no copies in or out.
// The FP64 cycle reproduces the reference V-cycle bit for bit.  The FP32 cycle (precision
// extension) runs the same steps in single precision.
#include <algorithm>
#include <cstring>
#include <limits>
#include <type_traits>

#include "mg_kernels.cuh"

namespace numa::gpu {

struct PoissonMG::Level {
    int n = 0;
    double h2inv = 0.0;
    double inv = 0.0;  // 1.0 / h2inv, as the reference forms it (poisson_mg.hpp:101)
    DeviceArray<double> x64, b64, bs64;
    DeviceArray<float> x32, b32, bs32;  // FP32 cycle (colour-split layout when n is odd)
    float* xs = nullptr;                // x32 past its front padding: the level's FP32 x
    float* cur32 = nullptr;             // the FP32 iterate of this level
};

namespace {

template <class T> T* xp(PoissonMG::Level& L);
template <> double* xp<double>(PoissonMG::Level& L) { return L.x64.p; }
template <> float* xp<float>(PoissonMG::Level& L) { return L.xs; }
template <class T> T* bp(PoissonMG::Level& L);
template <> double* bp<double>(PoissonMG::Level& L) { return L.b64.p; }
template <> float* bp<float>(PoissonMG::Level& L) { return L.b32.p; }
template <class T> T* bsp(PoissonMG::Level& L);
template <> double* bsp<double>(PoissonMG::Level& L) { return L.bs64.p; }
template <> float* bsp<float>(PoissonMG::Level& L) { return L.bs32.p; }

unsigned ew_grid(const Context& ctx, size_t N) {
    size_t want = (N + 255) / 256;
    size_t cap = static_cast<size_t>(ctx.sm_count) * 16;
    if (want > cap) want = cap;
    return static_cast<unsigned>(want < 1 ? 1 : want);
}

}  // namespace

PoissonMG::PoissonMG(Context& ctx, size_t n, int pre, int post, int precision, int max_levels)
    : ctx_(ctx), N0_(0), pre_(pre), post_(post), precision_(precision) {
    if (n == 0) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "PoissonMG requires a positive grid size");
    if (pre < 0 || post < 0) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "PoissonMG requires non-negative sweep counts");
    const size_t maxs = std::numeric_limits<size_t>::max();
    if (n > maxs / n || n * n > maxs / n) throw Status(NUMA_GPU_ERR_OVERFLOW, "PoissonMG cannot represent n^3");
    if (n > 65535) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "PoissonMG grid too large for one device");
    if (precision != NUMA_GPU_FP64 && precision != NUMA_GPU_FP32)
        throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "unknown precision");
    N0_ = n * n * n;
    if (precision == NUMA_GPU_FP32 && N0_ >= (size_t{1} << 31))
        throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "the FP32 V-cycle uses 32-bit indices: n^3 must be below 2^31");
    size_t m = n;
    double h2 = (static_cast<double>(n) + 1.0) * (static_cast<double>(n) + 1.0);
    for (;;) {
        auto L = std::make_unique<Level>();
        L->n = static_cast<int>(m);
        L->h2inv = h2;
        L->inv = 1.0 / h2;
        const size_t Nl = m * m * m;
        const bool finest = levels_.empty();
        if (precision == NUMA_GPU_FP64) {
            L->bs64.resize(Nl);
            if (!finest) {
                L->x64.resize(Nl);
                L->b64.resize(Nl);
            }
        } else {
            // x is padded by more than one plane of a colour on both sides, b and b h^2 at the end:
            // the FP32 kernels load every neighbour unconditionally (boundary values are then
            // replaced by zero with a select), and no load leaves the allocation
            const size_t pad = ((m * m - 1) / 2 + m + 2 + 31) / 32 * 32;
            L->x32.resize(Nl + 2 * pad);
            L->xs = L->x32.p + pad;
            L->b32.resize(Nl + 64);
            L->bs32.resize(Nl + 64);
        }
        levels_.push_back(std::move(L));
        if (m % 2 == 0 || m <= 1) break;
        if (max_levels > 0 && (int)levels_.size() >= max_levels) break;
        m = (m - 1) / 2;
        h2 /= 4.0;
    }
    if (levels_.size() > 1) {
        if (precision == NUMA_GPU_FP64) scratch_r_.resize(N0_);
        else scratch_r_.resize((N0_ + 1) / 2);  // N0 floats
    }
    // FP32: the levels of n <= 15 below the finest run as one CTA with shared-memory arrays
    if (precision == NUMA_GPU_FP32) {
        for (size_t l = 1; l < levels_.size(); ++l) {
            if (levels_[l]->n > 15) continue;
            if (levels_.size() - l > (size_t)kMaxTail) break;
            size_t elems = 0;
            // x, b, b h^2 and (Jacobian-aware tail) c h^2 of each level, and the residual scratch
            for (size_t m = l; m < levels_.size(); ++m) elems += 4 * (size_t)levels_[m]->n * levels_[m]->n * levels_[m]->n;
            elems += (size_t)levels_[l]->n * levels_[l]->n * levels_[l]->n;
            tail_smem_ = elems * sizeof(float);
            const int lim = std::min(set_dynamic_smem_limit(ctx_, k_mg_tail<float, true>),
                                     set_dynamic_smem_limit(ctx_, k_mg_tail<float, false>));
            if (tail_smem_ > (size_t)lim) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "PoissonMG tail exceeds shared memory");
            tail_l_ = l;
            break;
        }
    }
}

void PoissonMG::launch_tail32() {
    Level& L = *levels_[tail_l_];
    TailParams tp{};
    tp.levels = (int)(levels_.size() - tail_l_);
    for (int m = 0; m < tp.levels; ++m) {
        const Level& M = *levels_[tail_l_ + m];
        tp.n[m] = M.n;
        tp.h2inv[m] = M.h2inv;
        tp.inv[m] = M.inv;
        tp.six_h2inv[m] = 6.0 * M.h2inv;
    }
    tp.pre = pre_;
    tp.post = post_;
    const bool split = (L.n & 1) != 0;
    tp.half = split ? make_split(L.n).half : 0;
    for (int m = 0; m < kMaxTail; ++m) tp.c[m] = nullptr;
    if (coarse_jac_)
        for (int m = 0; m < tp.levels; ++m) tp.c[m] = cl_.p + cl_off_[tail_l_ + m];
    if (split) launch_pdl(k_mg_tail<float, true>, 1, 1024, tail_smem_, ctx_.stream, L.b32.p, L.bs32.p, L.xs, tp);
    else launch_pdl(k_mg_tail<float, false>, 1, 1024, tail_smem_, ctx_.stream, L.b32.p, L.bs32.p, L.xs, tp);
    ctx_.count_launch();
    L.cur32 = L.xs;
    ctx_.check_launch("mg tail (fp32)");
}

PoissonMG::~PoissonMG() {
    if (coarse_exec_) cudaGraphExecDestroy(coarse_exec_);
}

void PoissonMG::coarse_cycle() {
    if (coarse_exec_ && graph_jac_ != coarse_jac_) {  // captured in the other tail mode
        cudaGraphExecDestroy(coarse_exec_);
        coarse_exec_ = nullptr;
    }
    if (!coarse_exec_) {
        graph_jac_ = coarse_jac_;
        // no other thread may allocate or free (and so synchronise the device) during the capture
        std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
        const uint64_t before = ctx_.launches;
        NUMA_CUDA(cudaStreamBeginCapture(ctx_.stream, cudaStreamCaptureModeThreadLocal));
        cudaGraph_t graph = nullptr;
        try {
            if (precision_ == NUMA_GPU_FP64) cycle<double>(1);
            else cycle32(1);
        } catch (...) {
            cudaStreamEndCapture(ctx_.stream, &graph);
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            throw;
        }
        NUMA_CUDA(cudaStreamEndCapture(ctx_.stream, &graph));
        const cudaError_t e = cudaGraphInstantiate(&coarse_exec_, graph, 0);
        cudaGraphDestroy(graph);
        NUMA_CUDA(e);
        coarse_kernels_ = ctx_.launches - before;
        ctx_.launches = before;
    }
    NUMA_CUDA(cudaGraphLaunch(coarse_exec_, ctx_.stream));
    ctx_.count_launch(static_cast<unsigned>(coarse_kernels_));
}

template <class T>
void PoissonMG::cycle(size_t l) {
    Level& L = *levels_[l];
    const int n = L.n;
    const bool finest = (l == 0);
    T* x = finest ? static_cast<T*>(x0_) : xp<T>(L);
    const T* b = finest ? static_cast<const T*>(b0_) : bp<T>(L);
    const T* bs = finest ? static_cast<const T*>(bs0_) : bsp<T>(L);
    double* z = finest ? z0_ : nullptr;
    const size_t Nl = (size_t)n * n * n;
    cudaStream_t s = ctx_.stream;
    const dim3 blk(BX, BY);
    const dim3 cgrid(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, n);

    auto pass = [&](int colour, bool first, bool outz) {
        if (first && outz) launch_pdl(k_rbgs<T, true, true>, cgrid, blk, 0, s, x, bs, z, n, colour);
        else if (first) launch_pdl(k_rbgs<T, true, false>, cgrid, blk, 0, s, x, bs, nullptr, n, colour);
        else if (outz) launch_pdl(k_rbgs<T, false, true>, cgrid, blk, 0, s, x, bs, z, n, colour);
        else launch_pdl(k_rbgs<T, false, false>, cgrid, blk, 0, s, x, bs, nullptr, n, colour);
        ctx_.count_launch();
    };
    // order 0: colour 0 then 1; order 1: colour 1 then 0 (poisson_mg.hpp:103-106)
    auto sweep = [&](int order, bool first, bool outz) {
        const int c0 = order == 0 ? 0 : 1;
        pass(c0, first, outz);
        pass(1 - c0, false, outz);
    };

    if (l + 1 == levels_.size()) {
        if (n == 1) {
            launch_pdl(k_single<T>, 1, 1, 0, s, b, x, z, 6.0 * L.h2inv);
            ctx_.count_launch();
        } else {
            for (int sw = 0; sw < 30; ++sw) sweep(sw % 2, sw == 0, z != nullptr && sw == 29);
        }
        ctx_.check_launch("mg coarsest");
        return;
    }

    for (int sw = 0; sw < pre_; ++sw) sweep(0, sw == 0, false);
    if (pre_ == 0) NUMA_CUDA(cudaMemsetAsync(x, 0, Nl * sizeof(T), s));

    T* r = reinterpret_cast<T*>(scratch_r_.p);
    {
        const int ichunk = n >= 64 ? 8 : 1;
        const dim3 g((n + BX - 1) / BX, (n + BY - 1) / BY, (n + ichunk - 1) / ichunk);
        launch_pdl(k_residual<T>, g, blk, 0, s, x, b, r, n, ichunk, (T)L.h2inv);
        ctx_.count_launch();
    }
    Level& C = *levels_[l + 1];
    const int nc = C.n;
    {
        const dim3 g((nc + BX - 1) / BX, (nc + BY - 1) / BY, nc);
        launch_pdl(k_restrict<T>, g, blk, 0, s, r, bp<T>(C), bsp<T>(C), n, nc, C.inv);
        ctx_.count_launch();
    }
    ctx_.check_launch("mg restrict");
    if (l == 0) coarse_cycle();
    else cycle<T>(l + 1);
    if (post_ > 0) {
        const dim3 g(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, n);
        launch_pdl(k_prolong<T, true>, g, blk, 0, s, xp<T>(C), x, nc, n);
    } else {
        const dim3 g((n + BX - 1) / BX, (n + BY - 1) / BY, n);
        launch_pdl(k_prolong<T, false>, g, blk, 0, s, xp<T>(C), x, nc, n);
    }
    ctx_.count_launch();
    for (int sw = 0; sw < post_; ++sw) sweep(1, false, z != nullptr && sw == post_ - 1);
    if (z != nullptr && post_ == 0) {
        launch_pdl(k_to64, ew_grid(ctx_, Nl), 256, 0, s, reinterpret_cast<const float*>(x), z, Nl);
        ctx_.count_launch();
    }
    ctx_.check_launch("mg cycle");
}

// The FP32 cycle (precision extension): the same steps as cycle<double> in single precision.
// Levels of odd n (all but an even coarsest) keep x, b and b h^2 in the colour-split layout
// (mg_kernels.cuh), where every colour pass streams its own colour contiguously.  Three fusions
// remove whole passes over the finest level: the first smoothing pass of a split level (colour 0
// from x = 0) is written by the kernel that produces the level's right-hand side (the FP64 to
// FP32 conversion of r, or the restriction); the last pass of the cycle writes z in FP64 for
// both colours instead of storing x; and prolongation touches only the colour-0 fine points when
// post-smoothing follows.

// True when level l's first smoothing pass is fused into the producer of its right-hand side.
bool PoissonMG::first_fused32(size_t l) const {
    const Level& L = *levels_[l];
    if (!(L.n & 1) || l == tail_l_) return false;
    if (l + 1 == levels_.size()) return L.n > 1;  // coarsest: 30 sweeps, the first from x = 0
    return pre_ > 0;
}

void PoissonMG::cycle32(size_t l) {
    if (l == tail_l_) {
        launch_tail32();
        return;
    }
    Level& L = *levels_[l];
    const int n = L.n;
    const bool finest = (l == 0);
    const bool split = (n & 1) != 0;
    double* z = finest ? z0_ : nullptr;
    cudaStream_t s = ctx_.stream;
    const size_t Nl = (size_t)n * n * n;
    float* x = L.xs;
    const float* b = L.b32.p;
    const float* bs = L.bs32.p;
    const dim3 blk(BX, BY);
    const Split g = make_split(n);
    const dim3 cgrid(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, n);
    const bool fused_first = first_fused32(l);
    // pass(colour, first, last): last = the final pass of the cycle on the finest level
    auto pass = [&](int colour, bool first, bool last) {
        if (split) {
            if (first && fused_first) return;  // already written by the producer of b
            if (first) launch_pass_split<kPassFirst>(x, bs, nullptr, g, colour, s);
            else if (last && (z || (finest && z32_out_)))
                launch_pass_split<kPassLastZ>(x, bs, z, g, colour, s, finest ? z32_out_ : nullptr);
            else launch_pass_split<kPassFull>(x, bs, nullptr, g, colour, s);
        } else {
            if (first) launch_pdl(k_rbgs<float, true, false>, cgrid, blk, 0, s, x, bs, nullptr, n, colour);
            else launch_pdl(k_rbgs<float, false, false>, cgrid, blk, 0, s, x, bs, nullptr, n, colour);
        }
        ctx_.count_launch();
    };
    auto sweep = [&](int order, bool first, bool last) {
        const int c0 = order == 0 ? 0 : 1;
        pass(c0, first, false);
        pass(1 - c0, false, last);
    };
    // z from x when no pass wrote it
    auto out_z = [&]() {
        if (split) launch_pdl(k_to64_split, ew_grid(ctx_, Nl), 256, 0, s, x, z, (int)Nl, g.half);
        else launch_pdl(k_to64, ew_grid(ctx_, Nl), 256, 0, s, x, z, Nl);
        ctx_.count_launch();
    };
    L.cur32 = x;
    if (l + 1 == levels_.size()) {
        if (n == 1) {
            launch_pdl(k_single<float>, 1, 1, 0, s, b, x, z, 6.0 * L.h2inv);
            ctx_.count_launch();
        } else {
            for (int sw = 0; sw < 30; ++sw) sweep(sw % 2, sw == 0, sw == 29);
            if (z && !split) out_z();
        }
        ctx_.check_launch("mg coarsest (fp32)");
        return;
    }
    // a level with a coarser one below is odd, hence split
    for (int sw = 0; sw < pre_; ++sw) sweep(0, sw == 0, false);
    if (pre_ == 0) NUMA_CUDA(cudaMemsetAsync(x, 0, Nl * sizeof(float), s));
    float* r = reinterpret_cast<float*>(scratch_r_.p);
    Level& C = *levels_[l + 1];
    const int nc = C.n;
    const bool csplit = (nc & 1) != 0;
    {
        // two planes a thread sharing their i-neighbours (a four-plane march without the sharing took 80
        // registers)
        const dim3 rgd(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, (n + 1) / 2);
        // the finest level of an apply from an FP32 vector reads b = r32 itself (never copied, see apply)
        if (finest && in32_) launch_pdl(k_residual_split<true>, rgd, blk, 0, s, x, in32_, r, g, (float)L.h2inv);
        else launch_pdl(k_residual_split<false>, rgd, blk, 0, s, x, b, r, g, (float)L.h2inv);
        ctx_.count_launch();
    }
    const Split gc = make_split(nc);
    const dim3 rg((nc + BX - 1) / BX, (nc + BY - 1) / BY, nc);
    const dim3 rg2((nc + BX - 1) / BX, (nc + BY - 1) / BY, (nc + 1) / 2);  // two coarse planes a thread
    if (csplit && first_fused32(l + 1))
        launch_pdl(k_restrict_split<true>, rg2, blk, 0, s, r, C.b32.p, C.bs32.p, C.xs, n, nc, gc.half, (float)C.inv);
    else if (csplit)
        launch_pdl(k_restrict_split<false>, rg2, blk, 0, s, r, C.b32.p, C.bs32.p, C.xs, n, nc, gc.half, (float)C.inv);
    else
        launch_pdl(k_restrict<float>, rg, blk, 0, s, r, C.b32.p, C.bs32.p, n, nc, C.inv);
    ctx_.count_launch();
    if (l == 0) coarse_cycle();
    else cycle32(l + 1);
    const dim3 cg((nc + 1 + BX - 1) / BX, (nc + 1 + BY - 1) / BY, nc + 1);
    if (post_ > 0) {
        if (csplit) launch_pdl(k_prolong_split<true, false>, cg, blk, 0, s, C.cur32, x, nc, gc.half, n, g.half);
        else launch_pdl(k_prolong_split<false, false>, cg, blk, 0, s, C.cur32, x, nc, gc.half, n, g.half);
    } else {
        if (csplit) launch_pdl(k_prolong_split<true, true>, cg, blk, 0, s, C.cur32, x, nc, gc.half, n, g.half);
        else launch_pdl(k_prolong_split<false, true>, cg, blk, 0, s, C.cur32, x, nc, gc.half, n, g.half);
    }
    ctx_.count_launch();
    for (int sw = 0; sw < post_; ++sw) sweep(1, false, sw == post_ - 1);
    if (z && post_ == 0) out_z();
    ctx_.check_launch("mg cycle (fp32)");
}

// The FP32 cycle's finest level ends with a split pass that writes the output (odd n, a coarser
// level, post-smoothing): it can write z32 instead of z.
bool PoissonMG::supports_out32() const {
    return precision_ == NUMA_GPU_FP32 && (levels_[0]->n & 1) && levels_.size() > 1 && post_ > 0 && tail_l_ != 0;
}

void PoissonMG::apply32(const double* r, float* z32) {
    if (!supports_out32()) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "PoissonMG: no FP32 output for this hierarchy");
    z32_out_ = z32;
    try {
        apply(r, nullptr);
    } catch (...) {
        z32_out_ = nullptr;
        throw;
    }
    z32_out_ = nullptr;
}

void PoissonMG::apply32f(const float* r32, float* z32) {
    if (!supports_out32()) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "PoissonMG: no FP32 output for this hierarchy");
    z32_out_ = z32;
    in32_ = r32;
    try {
        apply(nullptr, nullptr);
    } catch (...) {
        z32_out_ = nullptr;
        in32_ = nullptr;
        throw;
    }
    z32_out_ = nullptr;
    in32_ = nullptr;
}

void PoissonMG::apply(const double* r, double* z) {
    Level& L0 = *levels_[0];
    const size_t N = N0_;
    if (precision_ == NUMA_GPU_FP64) {
        const double* b = r;
        if (r == z) {
            alias_b_.resize(N);
            dev_copy(ctx_, r, alias_b_.p, N);
            b = alias_b_.p;
        }
        launch_pdl(k_scale_in64, ew_grid(ctx_, N), 256, 0, ctx_.stream, b, L0.bs64.p, L0.inv, N);
        ctx_.count_launch();
        x0_ = z;
        b0_ = b;
        bs0_ = L0.bs64.p;
        z0_ = nullptr;
        cycle<double>(0);
    } else {
        auto scale_in = [&](auto rin) {
            using RT = std::remove_cv_t<std::remove_pointer_t<decltype(rin)>>;
            if (L0.n & 1) {
                const Split g = make_split(L0.n);
                const unsigned grid = ew_grid(ctx_, (size_t)g.half);
                // from an FP32 vector with a coarser level below, the residual reads b from the input itself
                const bool keep_b = !(std::is_same_v<RT, float> && levels_.size() > 1 && tail_l_ != 0);
                if (first_fused32(0) && !keep_b)
                    launch_pdl(k_scale_in32_split<true, RT, false>, grid, 256, 0, ctx_.stream, rin, L0.b32.p,
                               L0.bs32.p, L0.xs, (float)L0.inv, (int)N, g.half);
                else if (first_fused32(0))
                    launch_pdl(k_scale_in32_split<true, RT>, grid, 256, 0, ctx_.stream, rin, L0.b32.p, L0.bs32.p,
                               L0.xs, (float)L0.inv, (int)N, g.half);
                else
                    launch_pdl(k_scale_in32_split<false, RT>, grid, 256, 0, ctx_.stream, rin, L0.b32.p, L0.bs32.p,
                               L0.xs, (float)L0.inv, (int)N, g.half);
            } else {
                launch_pdl(k_scale_in32<RT>, ew_grid(ctx_, N), 256, 0, ctx_.stream, rin, L0.b32.p, L0.bs32.p,
                           (float)L0.inv, N);
            }
        };
        if (in32_) scale_in(in32_);
        else scale_in(r);
        ctx_.count_launch();
        z0_ = z;
        cycle32(0);
    }
    ctx_.check_launch("mg apply");
}

const float* PoissonMG::fine_b32() const { return levels_[0]->b32.p; }

namespace {

// cc = the full-weighting restriction of a natural-layout coefficient (restrict_coef_body, mg_kernels.cuh)
template <class TI>
__global__ void __launch_bounds__(BX* BY) k_restrict_coef(const TI* __restrict__ cf, float* __restrict__ cc, int nf,
                                                          int nc, int ichunk) {
    pdl_wait();
    pdl_trigger();
    restrict_coef_body(cf, cc, nf, nc, ichunk, blockIdx.x, blockIdx.y, blockIdx.z);
}

}  // namespace

void PoissonMG::set_coarse_coefficient(const double* c_fine, const float* c32_fine) {
    if (!supports_coarse_jacobian())
        throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "Jacobian-aware coarse levels need the FP32 cycle with a one-CTA tail");
    if (cl_off_.empty()) {
        size_t total = 0;
        cl_off_.assign(levels_.size(), 0);
        for (size_t l = 1; l < levels_.size(); ++l) {
            cl_off_[l] = total;
            total += (size_t)levels_[l]->n * levels_[l]->n * levels_[l]->n;
        }
        cl_.resize(total);
    }
    for (size_t l = 1; l < levels_.size(); ++l) {
        const int nf = levels_[l - 1]->n, nc = levels_[l]->n;
        const int ichunk = nc >= 64 ? 8 : (nc >= 16 ? 4 : 1);
        const dim3 g((nc + BX - 1) / BX, (nc + BY - 1) / BY, (nc + ichunk - 1) / ichunk);
        if (l == 1 && c32_fine)
            launch_pdl(k_restrict_coef<float>, g, dim3(BX, BY), 0, ctx_.stream, c32_fine, cl_.p + cl_off_[1], nf, nc,
                       ichunk);
        else if (l == 1)
            launch_pdl(k_restrict_coef<double>, g, dim3(BX, BY), 0, ctx_.stream, c_fine, cl_.p + cl_off_[1], nf, nc,
                       ichunk);
        else
            launch_pdl(k_restrict_coef<float>, g, dim3(BX, BY), 0, ctx_.stream, (const float*)(cl_.p + cl_off_[l - 1]),
                       cl_.p + cl_off_[l], nf, nc, ichunk);
        ctx_.count_launch();
    }
    ctx_.check_launch("mg coarse coefficient");
    coarse_jac_ = true;
}

double PoissonMG::time_finest_pass(int reps) {
    Level& L0 = *levels_[0];
    const int n = L0.n;
    const size_t N = N0_;
    const dim3 blk(BX, BY);
    const dim3 cgrid(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, n);
    cudaEvent_t a, b;
    NUMA_CUDA(cudaEventCreate(&a));
    NUMA_CUDA(cudaEventCreate(&b));
    float ms = 0.f;
    if (precision_ == NUMA_GPU_FP64) {
        DeviceArray<double> x(N);
        NUMA_CUDA(cudaMemsetAsync(x.p, 0, N * sizeof(double), ctx_.stream));
        NUMA_CUDA(cudaMemsetAsync(L0.bs64.p, 0, N * sizeof(double), ctx_.stream));
        launch_pdl(k_rbgs<double, false, false>, cgrid, blk, 0, ctx_.stream, x.p, L0.bs64.p, nullptr, n, 0);
        NUMA_CUDA(cudaEventRecord(a, ctx_.stream));
        for (int r = 0; r < reps; ++r)
            launch_pdl(k_rbgs<double, false, false>, cgrid, blk, 0, ctx_.stream, x.p, L0.bs64.p, nullptr, n, r & 1);
        NUMA_CUDA(cudaEventRecord(b, ctx_.stream));
        NUMA_CUDA(cudaEventSynchronize(b));
    } else {
        // the FP32 cycle's dominant kernel: one colour pass on the split layout (odd n)
        if (!(n & 1)) throw Status(NUMA_GPU_ERR_NOT_SUPPORTED, "the FP32 pass timing needs an odd grid");
        NUMA_CUDA(cudaMemsetAsync(L0.xs, 0, N * sizeof(float), ctx_.stream));
        NUMA_CUDA(cudaMemsetAsync(L0.bs32.p, 0, N * sizeof(float), ctx_.stream));
        const Split g = make_split(n);
        launch_pass_split<kPassFull>(L0.xs, L0.bs32.p, nullptr, g, 0, ctx_.stream);
        NUMA_CUDA(cudaEventRecord(a, ctx_.stream));
        for (int r = 0; r < reps; ++r) launch_pass_split<kPassFull>(L0.xs, L0.bs32.p, nullptr, g, r & 1, ctx_.stream);
        NUMA_CUDA(cudaEventRecord(b, ctx_.stream));
        NUMA_CUDA(cudaEventSynchronize(b));
    }
    ctx_.count_launch(reps + 1);
    NUMA_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    ctx_.check_launch("time_finest_pass");
    return reps > 0 ? ms / reps : 0.0;
}

}  // namespace numa::gpu
