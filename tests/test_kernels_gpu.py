"""GPU kernels against the oracle through the C ABI: stencils, BLAS-1, V-cycle.

Tolerances: the 7-point stencils, the V-cycle and axpy follow the reference's IEEE operation
order, so they are compared bit for bit, except where exp enters (CUDA's exp and the C
library's may differ by one ulp: bounded per element by a few ulps of lambda e^u).  Reductions
(dot, norm2) differ only in summation order: 1e-13 relative.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle_lib import make_point

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def _G():
    import numa_gpu
    return numa_gpu


def exp_tol(term, result, k=4.0):
    """Per-element bound for a difference caused by one-ulp exp rounding: k ulps of the exp
    term plus k ulps of the result (the final subtraction may then round the other way)."""
    return k * EPS * (np.abs(term) + np.abs(result)) + 1e-300


@pytest.mark.parametrize("n", [1, 2, 3, 6, 8, 15, 31, 33, 64])
@pytest.mark.parametrize("lam", [1.0, 6.0])
def test_bratu_operator(gpu, oracle, n, lam):
    G = _G()
    N = n ** 3
    u, v, w = make_point(N, 0.3), make_point(N, 1.0), make_point(N, 0.5)
    op = G.Bratu3D(gpu, n, lam)
    du, dv, dw, out = gpu.from_numpy(u), gpu.from_numpy(v), gpu.from_numpy(w), gpu.vec(N)
    c = lam * np.exp(u)
    op.eval(du, out)
    F = oracle.eval(n, lam, u)
    assert np.all(np.abs(out.numpy() - F) <= exp_tol(c, F))
    op.jvp(du, dv, out, G.ANALYTIC)
    J = oracle.jvp(n, lam, u, v, 0)
    assert np.all(np.abs(out.numpy() - J) <= exp_tol(c * v, J))
    op.d2(du, dw, out, G.ANALYTIC)
    D = oracle.d2(n, lam, u, w, 0)
    assert np.all(np.abs(out.numpy() - D) <= exp_tol(D, D))
    op.jacobi_diag(du, out)
    Dg = oracle.jacobi_diag(n, lam, u)
    assert np.all(np.abs(out.numpy() - Dg) <= exp_tol(c, Dg))
    # finite differences: the step h comes from reductions (summation order differs), and the
    # differences cancel, so the GPU's FD result is held to the accuracy of the oracle's own FD
    # result against the analytic derivative; at the reference test's size (n = 6) also to the
    # reference test's bounds (tests/test_operators.cpp:46, :60)
    op.jvp(du, dv, out, G.FD)
    Jfd = oracle.jvp(n, lam, u, v, 1)
    assert rel_err(out.numpy(), J) <= 2 * rel_err(Jfd, J) + 1e-9
    op.d2(du, dw, out, G.FD)
    Dfd = oracle.d2(n, lam, u, w, 1)
    assert rel_err(out.numpy(), D) <= 2 * rel_err(Dfd, D) + 1e-7
    if n <= 8:
        op.jvp(du, dv, out, G.FD)
        assert rel_err(out.numpy(), J) < 1e-6
        op.d2(du, dw, out, G.FD)
        assert rel_err(out.numpy(), D) < 1e-4


def test_bratu_operator_golden(gpu, ref_vectors):
    """The reference's own outputs on its test inputs (n = 6, 8)."""
    G = _G()
    for n in (6, 8):
        N = n ** 3
        u, v, w = ref_vectors[f"op_n{n}_u"], ref_vectors[f"op_n{n}_v"], make_point(N, 0.5)
        op = G.Bratu3D(gpu, n, 1.0)
        du, dv, dw, out = gpu.from_numpy(u), gpu.from_numpy(v), gpu.from_numpy(w), gpu.vec(N)
        op.eval(du, out)
        F = ref_vectors[f"op_n{n}_eval"]
        assert np.all(np.abs(out.numpy() - F) <= exp_tol(np.exp(u), F))
        op.jvp(du, dv, out)
        assert rel_err(out.numpy(), ref_vectors[f"op_n{n}_jvp"]) < 1e-15
        op.d2(du, dw, out)
        assert rel_err(out.numpy(), ref_vectors[f"op_n{n}_d2"]) < 1e-15


def test_blas1(gpu):
    rng = np.random.default_rng(1234)
    for N in (1, 7, 1000, 300_007):
        a, b = rng.uniform(-1, 1, N), rng.uniform(-1, 1, N)
        da, db = gpu.from_numpy(a), gpu.from_numpy(b)
        assert da.dot(db) == pytest.approx(float(np.dot(a, b)), rel=1e-12, abs=1e-13)
        assert da.norm2() == pytest.approx(float(np.linalg.norm(a)), rel=1e-13)
        db.axpy(-0.7, da)
        assert np.array_equal(db.numpy(), b + (-0.7) * a)  # y += a*x, no contraction
    z = gpu.vec(0)
    assert z.norm2() == 0.0


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 15, 16, 21, 31, 63])
@pytest.mark.parametrize("pre_post", [(2, 2), (1, 1), (0, 2), (2, 0), (3, 1)])
def test_vcycle_bit_exact(gpu, oracle, n, pre_post):
    """One FP64 V-cycle equals the reference algorithm bit for bit (no reductions inside)."""
    G = _G()
    pre, post = pre_post
    N = n ** 3
    r = make_point(N, 1.0)
    mg = G.PoissonMG(gpu, n, pre, post)
    assert mg.levels() == oracle.mg_levels(n, pre, post)
    dr, dz = gpu.from_numpy(r), gpu.vec(N)
    dz.fill(123.0)  # garbage in z must not leak into the result
    mg(dr, dz)
    assert np.array_equal(dz.numpy(), oracle.mg_apply(n, r, pre, post))
    mg(dr, dz)  # a second application reuses the hierarchy's arrays
    assert np.array_equal(dz.numpy(), oracle.mg_apply(n, r, pre, post))


def test_vcycle_golden_and_random(gpu, oracle, ref_vectors):
    G = _G()
    mg = G.PoissonMG(gpu, 15)
    dz = gpu.vec(15 ** 3)
    mg(gpu.from_numpy(make_point(15 ** 3, 1.0)), dz)
    assert np.array_equal(dz.numpy(), ref_vectors["mg_n15_z"])
    rng = np.random.default_rng(7)
    for n in (31, 127):
        r = rng.uniform(-1, 1, n ** 3) * 10.0 ** rng.uniform(-3, 3, n ** 3)
        mg = G.PoissonMG(gpu, n)
        dz = gpu.vec(n ** 3)
        mg(gpu.from_numpy(r), dz)
        assert np.array_equal(dz.numpy(), oracle.mg_apply(n, r))


def test_vcycle_residual_reduction(gpu):
    """tests/test_operators.cpp:189-205: one V-cycle reduces ||b - A z|| below 0.5 ||b||."""
    G = _G()
    n = 15
    mg = G.PoissonMG(gpu, n)
    assert mg.levels() == 4
    b = gpu.from_numpy(make_point(n ** 3, 1.0))
    z, Az, zero = gpu.vec(n ** 3), gpu.vec(n ** 3), gpu.vec(n ** 3)
    mg(b, z)
    lap = G.Bratu3D(gpu, n, 0.0)  # jvp at lambda = 0 is -Laplacian_h
    lap.jvp(zero, z, Az)
    Az.axpy(-1.0, b)
    assert Az.norm2() < 0.5 * b.norm2()


def test_vcycle_aliasing(gpu, oracle):
    """r and z may be the same vector: the result is the V-cycle of the input."""
    G = _G()
    n = 15
    r = make_point(n ** 3, 1.0)
    mg = G.PoissonMG(gpu, n)
    v = gpu.from_numpy(r)
    mg(v, v)
    assert np.array_equal(v.numpy(), oracle.mg_apply(n, r))


def test_vcycle_fp32(gpu, oracle):
    G = _G()
    for n in (15, 63):
        r = make_point(n ** 3, 1.0)
        mg = G.PoissonMG(gpu, n, precision=G.FP32)
        dz = gpu.vec(n ** 3)
        mg(gpu.from_numpy(r), dz)
        assert rel_err(dz.numpy(), oracle.mg_apply(n, r)) < 5e-6


def test_mg_errors(gpu):
    G = _G()
    with pytest.raises(G.NumaGPUError) as e:
        G.PoissonMG(gpu, 0)
    assert e.value.code == 1  # invalid_argument (poisson_mg.hpp:29-32)
    with pytest.raises(G.NumaGPUError) as e:
        G.PoissonMG(gpu, 7, -1, 2)
    assert e.value.code == 1  # (poisson_mg.hpp:33-36)
    mg = G.PoissonMG(gpu, 7)
    with pytest.raises(G.NumaGPUError) as e:
        mg(gpu.vec(8), gpu.vec(8))
    assert e.value.code == 1  # residual of incompatible size (poisson_mg.hpp:71-74)


def test_max_levels_extension(gpu, oracle):
    G = _G()
    mg = G.PoissonMG(gpu, 31, max_levels=2)
    assert mg.levels() == 2
    dz = gpu.vec(31 ** 3)
    mg(gpu.from_numpy(make_point(31 ** 3, 1.0)), dz)
    assert np.all(np.isfinite(dz.numpy()))


def _ulp_diff(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """|a - b| in units of the last place, for finite positive doubles (ordered bit patterns)."""
    ia, ib = a.view(np.int64), b.view(np.int64)
    return np.abs(ia - ib)


def test_exp_table_driven(gpu):
    """The residual kernels' e^x (Tang's table-driven method) against the host C library and
    CUDA's exp: within 1 ulp everywhere, exact at the special values."""
    import numa_gpu as G
    rng = np.random.default_rng(1234)
    x = np.concatenate([
        rng.uniform(-707.9, 707.9, 600_000),
        rng.uniform(-2.0, 2.0, 600_000),            # the Bratu range
        rng.uniform(-1e-6, 1e-6, 50_000),
        np.arange(-22000, 22000) * (np.log(2) / 32),  # table boundaries
        np.array([0.0, -0.0, 1e-300, -1e-300, 707.99, -707.99, 708.0, -708.0, 709.7, -745.2, -746.0, 710.0,
                  np.inf, -np.inf, np.nan]),
    ])
    xv, out, ref = gpu.from_numpy(x), gpu.vec(x.size), gpu.vec(x.size)
    G.diag_exp(xv, out, ref)
    got, cuda = out.numpy(), ref.numpy()
    host = np.exp(x)
    fin = np.isfinite(host) & (host > 0) & (host >= np.finfo(float).tiny)
    assert _ulp_diff(got[fin], host[fin]).max() <= 1
    assert _ulp_diff(got[fin], cuda[fin]).max() <= 2
    # most results are correctly rounded (equal to the host's)
    assert np.mean(got[fin] == host[fin]) > 0.99
    special = ~fin
    assert np.array_equal(got[special], cuda[special], equal_nan=True)
    assert np.all(got[x == 0.0] == 1.0)


def test_fd_quotient_division_correctly_rounded(gpu):
    """The finite-difference quotients divide by h (or h^2) through RN(1/h) and Markstein's
    correction: every quotient must equal the IEEE division bit for bit, for step sizes of the
    operators' range and for arbitrary divisors, including significands of all ones, zeros,
    subnormals, huge values, infinities and NaN."""
    import numa_gpu as G
    rng = np.random.default_rng(77)
    M = 400_000
    a = np.concatenate([
        rng.standard_normal(M) * 10.0 ** rng.uniform(-30, 30, M),
        rng.uniform(-1, 1, M) * 2.0 ** rng.integers(-1074, 1023, M),
        np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                  1.7976931348623157e308, -1.7976931348623157e308, 1.0, np.nextafter(2.0, 0)]),
    ])
    av, out = gpu.from_numpy(a), gpu.vec(a.size)
    divisors = [1.4901161193847656e-08, 2.2204460492503131e-16, 3.7e-9, 1.2e-17, np.nextafter(2.0, 0),
                -np.nextafter(1.0, 0), 3.0, 0.1, 1e-300, 1e300, 2.0 ** -960, 2.0 ** 960, 5e-324, 0.0,
                np.inf, np.nan]
    divisors += list(rng.uniform(1, 2, 6) * 2.0 ** rng.integers(-1000, 1000, 6))
    with np.errstate(all="ignore"):
        for b in divisors:
            G.diag_div(av, b, out)
            want = a / b
            got = out.numpy()
            assert np.array_equal(got.view(np.int64), want.view(np.int64)) or \
                np.array_equal(got, want, equal_nan=True), b
            bad = (got.view(np.int64) != want.view(np.int64)) & ~(np.isnan(got) & np.isnan(want))
            assert not bad.any(), (b, a[bad][:4], got[bad][:4], want[bad][:4])
