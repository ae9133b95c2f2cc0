// The reference's own nonlinear drivers and GMRES (namespace numa::op), instantiated unchanged
// with the GPU operator and preconditioner of numa/gpu/numa_gpu.hpp.  This program is compiled
// and linked against libnuma_gpu.so where the reference headers are present
// (tests/test_cpp_adaptor.py); run on a GPU host, each operator call moves its vectors to and
// from the GPU.
#include <numa/linalg/gmres.hpp>
#include <numa/methods/krylov_newton.hpp>
#include <numa/methods/tf_chebyshev_2018.hpp>

#include "numa/gpu/numa_gpu.hpp"

#include <cstdio>

static_assert(numa::op::NonlinearOperator<numa::gpu::Bratu3D>);
static_assert(numa::op::SecondOrderOperator<numa::gpu::Bratu3D>);

int main() {
    numa::gpu::Context ctx(0);
    numa::gpu::Bratu3D f(ctx, 16, 1.0);
    const numa::op::DVec x0(f.size(), 0.0);
    auto pc = numa::gpu::Provider::poisson_mg(ctx, 16);
    const auto nk = numa::op::newton_krylov(f, x0, numa::op::KrylovParams{}, pc);
    const auto ch = numa::op::chebyshev_inexact(f, x0, numa::op::KrylovParams{}, pc);
    const auto tf = numa::op::tf_chebyshev_2018(f, x0, numa::op::KrylovParams{}, pc);
    numa::gpu::PoissonMG mg(ctx, 15);
    numa::op::DVec b(15 * 15 * 15, 1.0), z(b.size(), 0.0);
    auto apply = [&](const numa::op::DVec& v, numa::op::DVec& out) { out = v; };
    const auto g = numa::op::gmres(apply, mg, b, z, 1e-8, 30, 100);
    std::printf("nk %zu %zu %zu cheb %zu %zu %zu tf %zu gmres %zu\n", nk.iters, nk.n_JVP, nk.n_prec, ch.iters,
                ch.n_JVP, ch.n_prec, tf.iters, g.iters);
    return nk.converged && ch.converged ? 0 : 1;
}
