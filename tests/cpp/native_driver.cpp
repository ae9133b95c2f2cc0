// A C++ caller of the native GPU drivers through numa/gpu/numa_gpu.hpp only (no reference
// headers): Bratu3D 31^3, lambda = 6, rtol 1e-10, GMRES(30), MG V(2,2); prints the counts and
// max(u), then the mixed path's counts and its distance to that solve.  Built and run by
// tests/test_cpp_adaptor.py on a GPU host.
#include "numa/gpu/numa_gpu.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>

int main(int argc, char** argv) {
    const std::size_t n = argc > 1 ? std::strtoul(argv[1], nullptr, 10) : 31;
    numa::gpu::Context ctx(0);
    numa::gpu::Bratu3D f(ctx, n, 6.0);
    auto pc = numa::gpu::Provider::poisson_mg(ctx, n);
    numa::gpu::KrylovParams p;
    p.rtol_nl = 1e-10;
    p.gmres_restart = 30;
    const auto r = numa::gpu::newton_krylov(f, numa::gpu::DVec(f.size(), 0.0), p, &pc);
    const auto c = numa::gpu::chebyshev_inexact(f, numa::gpu::DVec(f.size(), 0.0), p, &pc);
    std::printf("nk %zu %zu %zu %zu %d %.17g\n", r.iters, r.n_F, r.n_JVP, r.n_prec, (int)r.converged,
                *std::max_element(r.x.begin(), r.x.end()));
    std::printf("cheb %zu %zu %zu %zu %zu %d\n", c.iters, c.n_F, c.n_JVP, c.n_D2, c.n_prec, (int)c.converged);
    // the benchmark's mixed path through the same adaptor: FGMRES, FP32 V-cycle with the Jacobian on its
    // coarse levels, FP32 products (of FP64 accuracy in the tight linear solves); its distance to the FP64 solve
    auto pj = numa::gpu::Provider::jacobian_mg(ctx, n);
    numa::gpu::KrylovParams q = p;
    q.flexible = 1;
    q.jvp_precision = NUMA_GPU_FP32;
    q.orth = NUMA_GPU_ORTH_CGS1;
    q.jvp_tight = 1;
    const auto m = numa::gpu::newton_krylov(f, numa::gpu::DVec(f.size(), 0.0), q, &pj);
    double num = 0.0, den = 0.0;
    for (std::size_t i = 0; i < r.x.size(); ++i) {
        num += (m.x[i] - r.x[i]) * (m.x[i] - r.x[i]);
        den += r.x[i] * r.x[i];
    }
    std::printf("mixed %zu %zu %d %.3e\n", m.iters, m.n_lin_iters, (int)m.converged, std::sqrt(num / den));
    // error path: PoissonMG rejects n = 0 with std::invalid_argument, as the reference does
    try {
        numa::gpu::PoissonMG bad(ctx, 0);
        return 2;
    } catch (const std::invalid_argument&) {
    }
    return r.converged && c.converged && m.converged ? 0 : 1;
}
