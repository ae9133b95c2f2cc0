// batch.cu — many independent Bratu3D solves on one GPU (instances of uneven grid size and
// lambda, the batched configuration): a native executor of `workers` host threads, each with its
// own context (device stream, reduction scratch) and its own operators, multigrid hierarchies and
// solver workspaces, kept per grid size and reused across instances (lambda is a parameter of the
// kernels, so an operator serves every lambda).  The GPU interleaves the workers' streams, which
// is what the small grids need: a 31^3 or 63^3 solve alone leaves most of the 152 SMs idle.
// Instances are taken largest first (longest-processing-time order) from a shared counter.  The
// executor keeps its workers' device state between batches, so a second batch allocates nothing.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "numa_internal.hpp"

namespace numa::gpu {

// One worker's device state, kept between batches: its context and, per grid size, the operator,
// the multigrid provider and the iterate.
struct BatchWorker {
    explicit BatchWorker(int device) : ctx(device) {}
    Context ctx;
    std::map<size_t, std::unique_ptr<Bratu3D>> ops;
    std::map<size_t, std::unique_ptr<Provider>> pcs;
    std::map<size_t, DeviceArray<double>> xs;
};

BatchExecutor::BatchExecutor(int device, int workers) : device_(device) {
    const int nw = std::max(1, workers);
    for (int w = 0; w < nw; ++w) workers_.push_back(std::make_unique<BatchWorker>(device));
    active_ = nw;
}

void BatchExecutor::set_active(int w) {
    if (w < 1 || w > (int)workers_.size()) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "worker count out of range");
    active_ = w;
}

int BatchExecutor::autotune(const numa_batch_instance* inst, size_t count, int method, int mg_precision,
                            const numa_krylov_params* params, const int* candidates, int ncand, double* seconds) {
    if (ncand < 1 || !candidates) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "no candidate worker counts");
    std::vector<numa_batch_result> res(count);
    int best = -1;
    double best_t = 0.0;
    for (int c = 0; c < ncand; ++c) {
        set_active(candidates[c]);
        double t = 0.0;
        solve(inst, count, method, mg_precision, params, res.data(), &t);  // sets the workers up
        solve(inst, count, method, mg_precision, params, res.data(), &t);
        if (seconds) seconds[c] = t;
        if (best < 0 || t < best_t) {
            best = candidates[c];
            best_t = t;
        }
    }
    set_active(best);
    return best;
}

BatchExecutor::~BatchExecutor() = default;

void BatchExecutor::solve(const numa_batch_instance* inst, size_t count, int method, int mg_precision,
                          const numa_krylov_params* params, numa_batch_result* results, double* wall_seconds) {
    std::vector<size_t> order(count);
    std::iota(order.begin(), order.end(), size_t{0});
    std::stable_sort(order.begin(), order.end(), [inst](size_t a, size_t b) { return inst[a].n > inst[b].n; });
    std::atomic<size_t> next{0};
    std::mutex err_mutex;
    int err_code = 0;
    std::string err_msg;
    const auto t0 = std::chrono::steady_clock::now();
    auto work = [&](BatchWorker& wk) {
        try {
            NUMA_CUDA(cudaSetDevice(device_));
            Context& ctx = wk.ctx;
            for (;;) {
                const size_t k = next.fetch_add(1);
                if (k >= count) break;
                {
                    std::lock_guard<std::mutex> lk(err_mutex);
                    if (err_code) break;
                }
                const size_t i = order[k];
                const size_t n = inst[i].n;
                auto& op = wk.ops[n];
                if (!op) op = std::make_unique<Bratu3D>(ctx, n, inst[i].lambda);
                op->set_lambda(inst[i].lambda);
                auto& pc = wk.pcs[(n << 1) | (size_t)mg_precision];
                if (!pc) pc = make_mg_provider(ctx, n, 2, 2, mg_precision, 0);
                auto& x = wk.xs[n];
                x.resize(n * n * n);
                dev_fill(ctx, x.p, 0.0, n * n * n);
                KrylovParams kp = params_from_c(params);
                numa_krylov_result r;
                std::memset(&r, 0, sizeof(r));
                if (method == NUMA_GPU_METHOD_NK) {
                    newton_krylov(*op, x.p, kp, pc.get(), r);
                } else if (method == NUMA_GPU_METHOD_TF2018) {
                    tf_chebyshev_2018(*op, x.p, kp, pc.get(), r);
                } else {
                    if (method == NUMA_GPU_METHOD_CHEB_REC) kp.recycle = true;
                    chebyshev_inexact(*op, x.p, kp, pc.get(), r);
                }
                numa_batch_result& o = results[i];
                o.converged = r.converged;
                o.status = 0;
                o.iters = r.iters;
                o.n_F = r.n_F;
                o.n_JVP = r.n_JVP;
                o.n_lin_iters = r.n_lin_iters;
                o.n_prec = r.n_prec;
                o.res_rel = r.res0 > 0.0 ? r.res / r.res0 : r.res;
                o.seconds = r.t_total;
            }
            ctx.sync();
        } catch (const Status& s) {
            std::lock_guard<std::mutex> lk(err_mutex);
            if (!err_code) {
                err_code = s.code;
                err_msg = s.what();
            }
        } catch (const std::exception& e) {
            std::lock_guard<std::mutex> lk(err_mutex);
            if (!err_code) {
                err_code = NUMA_GPU_ERR_CUDA;
                err_msg = e.what();
            }
        }
    };
    const size_t nw = std::min((size_t)active_, std::max<size_t>(count, 1));
    std::vector<std::thread> threads;
    threads.reserve(nw);
    for (size_t w = 0; w < nw; ++w) threads.emplace_back(work, std::ref(*workers_[w]));
    for (auto& t : threads) t.join();
    if (wall_seconds) *wall_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (err_code) throw Status(err_code, "batched solve: " + err_msg);
}

}  // namespace numa::gpu
