"""Mixed-precision kernels (an extension of the reference path) against a numpy float32
restatement of the same arithmetic: the FP32 V-cycle (fused red-black sweeps, integer
FP64<->FP32 conversions) and the FP32 Jacobian-vector product must match it bit for bit; numpy's
float32 operations are IEEE single precision, and x/6 is correctly rounded in both."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle_lib import make_point

pytestmark = pytest.mark.gpu

F = np.float32
NOT_SUPPORTED = 8  # NUMA_GPU_ERR_NOT_SUPPORTED


def _G():
    import numa_gpu
    return numa_gpu


def shifted(x, axis, d):
    """x shifted so that out[i] = x[i + d] along axis, zero outside (Dirichlet)."""
    out = np.zeros_like(x)
    n = x.shape[axis]
    src = [slice(None)] * 3
    dst = [slice(None)] * 3
    if d > 0:
        src[axis], dst[axis] = slice(d, n), slice(0, n - d)
    else:
        src[axis], dst[axis] = slice(0, n + d), slice(-d, n)
    out[tuple(dst)] = x[tuple(src)]
    return out


def colour_mask(n):
    i, j, k = np.indices((n, n, n))
    return (i + j + k) & 1


def rb_pass(x, bs, colour, mask):
    acc = bs.copy()
    for axis in (0, 1, 2):
        acc = acc + shifted(x, axis, -1)
        acc = acc + shifted(x, axis, +1)
    new = acc / F(6)
    x = x.copy()
    x[mask == colour] = new[mask == colour]
    return x


def vcycle32(r64, n, pre=2, post=2):
    """The FP32 V-cycle of this library (poisson_mg.cu cycle32) in numpy float32."""
    levels = []
    m, h2 = n, (n + 1.0) ** 2
    while True:
        levels.append((m, h2, 1.0 / h2))
        if m % 2 == 0 or m <= 1:
            break
        m, h2 = (m - 1) // 2, h2 / 4.0
    w = np.array([0.25, 0.5, 0.25], dtype=F)

    def cycle(l, b, bs):
        m, h2, _ = levels[l]
        mask = colour_mask(m)
        x = np.zeros((m, m, m), F)
        if l + 1 == len(levels):
            if m == 1:
                return np.array([[[F(np.float64(b[0, 0, 0]) / (6.0 * h2))]]], F)
            for sw in range(30):
                c0 = sw % 2
                x = rb_pass(x, bs, c0, mask)
                x = rb_pass(x, bs, 1 - c0, mask)
            return x
        for _ in range(pre):
            x = rb_pass(x, bs, 0, mask)
            x = rb_pass(x, bs, 1, mask)
        s = F(6) * x
        for axis in (0, 1, 2):
            s = s - shifted(x, axis, -1)
            s = s - shifted(x, axis, +1)
        r = b - F(h2) * s
        mc, _, invc = levels[l + 1]
        acc = np.zeros((mc, mc, mc), F)
        for a in range(3):
            for bb in range(3):
                for c in range(3):
                    acc = acc + (w[a] * w[bb] * w[c]) * r[a:a + 2 * mc:2, bb:bb + 2 * mc:2, c:c + 2 * mc:2]
        xc = cycle(l + 1, acc, acc * F(invc))
        # trilinear prolongation at colour-0 points (post > 0), summed i outer, j, k inner over each
        # fine index's one or two coarse neighbours; a missing neighbour is a zero term with weight
        # zero (acc + 0 is exact, so the slots keep the kernel's order)
        tix = np.full((2, m), mc)
        tw = np.zeros((2, m), F)
        for f in range(m):
            if f % 2 == 1:
                lst = [((f - 1) // 2, F(1))]
            else:
                lst = [(c, F(0.5)) for c in (f // 2 - 1, f // 2) if 0 <= c < mc]
            for t, (c, wt) in enumerate(lst):
                tix[t, f], tw[t, f] = c, wt
        xcp = np.zeros((mc + 1,) * 3, F)
        xcp[:mc, :mc, :mc] = xc
        acc2 = np.zeros((m, m, m), F)
        for ti in range(2):
            for tj in range(2):
                for tk in range(2):
                    wt = tw[ti][:, None, None] * tw[tj][None, :, None] * tw[tk][None, None, :]
                    acc2 = acc2 + wt * xcp[np.ix_(tix[ti], tix[tj], tix[tk])]
        pr = np.where(mask == 0, acc2, F(0)) if post > 0 else acc2
        x = x + pr
        for _ in range(post):
            x = rb_pass(x, bs, 1, mask)
            x = rb_pass(x, bs, 0, mask)
        return x

    b = r64.reshape(n, n, n).astype(F)
    bs = b * F(levels[0][2])
    return cycle(0, b, bs).astype(np.float64).ravel()


@pytest.mark.parametrize("n", [1, 3, 7, 15, 16, 21, 23, 31, 63, 127, 255])
def test_fp32_vcycle_bit_exact(gpu, n):
    G = _G()
    N = n ** 3
    rng = np.random.default_rng(n)
    r = make_point(N, 1.0) + rng.uniform(-1e-3, 1e-3, N)
    mg = G.PoissonMG(gpu, n, precision=G.FP32)
    z = gpu.vec(N)
    z.fill(5.0)
    want = vcycle32(r, n)
    for _ in range(2):
        mg(gpu.from_numpy(r), z)
        assert np.array_equal(z.numpy(), want)


@pytest.mark.parametrize("n", [2, 6, 33, 64])
def test_fp32_jvp_bit_exact(gpu, n):
    G = _G()
    N = n ** 3
    rng = np.random.default_rng(3 * n)
    u = make_point(N, 0.3)
    v = rng.uniform(-1, 1, N) * 10.0 ** rng.integers(-30, 30, N)
    v[:5] = [0.0, -0.0, 1e-300, -3.5e38, 2.0 ** -130]  # zero, underflow, overflow, float subnormal
    op = G.Bratu3D(gpu, n, 6.0)
    out = gpu.vec(N)
    op.jvp(gpu.from_numpy(u), gpu.from_numpy(v), out, G.ANALYTIC_FP32)
    # numpy float32 restatement; c = RN32(lambda e^u) with numpy's exp (CUDA's may differ by an
    # ulp in FP64, which moves the FP32 rounding only for values within an ulp of a float
    # rounding boundary: probability ~2^-29 per element)
    c = 6.0 * np.exp(u)
    with np.errstate(over="ignore", invalid="ignore"):
        vf = v.reshape(n, n, n).astype(F)
        s = F(6) * vf
        for axis in (0, 1, 2):
            s = s - shifted(vf, axis, -1)
            s = s - shifted(vf, axis, +1)
        want = (F((n + 1.0) ** 2) * s - c.reshape(n, n, n).astype(F) * vf).astype(np.float64).ravel()
    got = out.numpy()
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    assert same.all(), np.flatnonzero(~same)[:10]


@pytest.mark.parametrize("n", [5, 31, 64])
@pytest.mark.parametrize("smooth", [False, True])
def test_fp32_input_product_to_fp64_accuracy(gpu, n, smooth):
    """The product the mixed path's tight linear solves take (jvp_tight): F'(u) RN32(v) by a
    double-FP32 stencil with the FP64 coefficient, against the FP64 product of the same FP32 values
    in numpy (sums of FP32 values of these magnitudes are exact in FP64).  Bound: 2^-44 of the
    stencil's largest partial sum plus a few FP64 roundings of c v and the result.  On a smooth v,
    whose Laplacian cancels, FP32 arithmetic misses that accuracy by orders of magnitude."""
    G = _G()
    N = n ** 3
    u = make_point(N, 0.3)
    if smooth:
        t = np.arange(1, n + 1) / (n + 1.0)
        s1 = np.sin(np.pi * t)
        v = (s1[:, None, None] * s1[None, :, None] * s1[None, None, :]).ravel()
    else:
        v = np.random.default_rng(n).uniform(-1, 1, N)
    op = G.Bratu3D(gpu, n, 6.0)
    out = gpu.vec(N)
    op.jvp(gpu.from_numpy(u), gpu.from_numpy(v), out, G.ANALYTIC_FP32X)
    vf = v.astype(F).astype(np.float64).reshape(n, n, n)
    h2 = (n + 1.0) ** 2
    s = 6.0 * vf
    mag = 6.0 * np.abs(vf)
    for axis in (0, 1, 2):
        for d in (-1, 1):
            nb = shifted(vf, axis, d)
            s = s - nb
            mag = mag + np.abs(nb)
    c = 6.0 * np.exp(u.reshape(n, n, n))
    want = h2 * s - c * vf
    tol = (2.0 ** -44 * h2 * mag + 2.0 ** -50 * (np.abs(c * vf) + np.abs(want))).ravel()
    want = want.ravel()
    got = out.numpy()
    bad = np.abs(got - want) > tol
    assert not bad.any(), (np.flatnonzero(bad)[:10], np.abs(got - want)[bad][:5], tol[bad][:5])
    if smooth and n >= 31:
        out32 = gpu.vec(N)
        op.jvp(gpu.from_numpy(u), gpu.from_numpy(vf.ravel()), out32, G.ANALYTIC_FP32)
        ex = rel_err(got, want)
        e32 = rel_err(out32.numpy(), want)
        assert ex < 1e-13 and e32 > 1e3 * ex, (ex, e32)


def _exact_lap_sum(u):
    """6u - (the six neighbours) of every point, the exact sum rounded once (math.fsum)."""
    import math
    n = u.shape[0]
    nb = [shifted(u, axis, d).ravel() for axis in (0, 1, 2) for d in (-1, 1)]
    c = u.ravel()
    return np.array([math.fsum((c[p],) * 6 + tuple(-a[p] for a in nb)) for p in range(n ** 3)]), nb


@pytest.mark.parametrize("n,case", [(7, "point"), (31, "point"), (31, "wide"), (20, "special"), (64, "point")])
def test_mixed_evaluation_fixed_point_sum(gpu, n, case):
    """The mixed path's residual evaluation forms 6u - (six neighbours) in 64-bit fixed point and
    rounds it once, then F = h^-2 s - lambda e^u with one rounding.  Bound against the exactly
    rounded sum (fsum): h^-2 (7 2^-56 max|values| + 2^-52 |S|) for the sum, an ulp of lambda e^u
    (the table-driven exponential against numpy's), half an ulp of F.  Cases: the reference's test
    point, magnitudes spread over 25 decades (deep truncation of the aligned values), and zeros,
    signed zeros and subnormals (a subnormal result takes the FP64 chain)."""
    G = _G()
    N = n ** 3
    rng = np.random.default_rng(n)
    if case == "point":
        u = make_point(N, 0.3)
    elif case == "wide":
        u = rng.uniform(-1, 1, N) * 10.0 ** rng.integers(-20, 2, N)
    else:
        u = rng.uniform(-1, 1, N) * 1e-3
        u[: N // 4] = 0.0
        u[N // 4: N // 3] = -0.0
        u[N // 3: N // 2] = rng.uniform(-1, 1, N // 2 - N // 3) * 1e-310  # subnormals
    lam = 2.0 ** -10  # the smallest lambda of the scaled exp table: lambda e^u small beside the stencil
    op = G.Bratu3D(gpu, n, lam)
    out, out64 = gpu.vec(N), gpu.vec(N)
    nrm = op.eval_as(gpu.from_numpy(u), out, G.FP32)
    u3 = u.reshape(n, n, n)
    S, nb = _exact_lap_sum(u3)
    h2 = (n + 1.0) ** 2
    e = lam * np.exp(u)
    want = h2 * S - e
    vmax = np.maximum.reduce([np.abs(u)] + [np.abs(a) for a in nb])
    tol = h2 * (7 * 2.0 ** -56 * vmax + 2.0 ** -52 * np.abs(S)) + 2.0 ** -51 * np.abs(e) + 2.0 ** -52 * np.abs(want)
    got = out.numpy()
    bad = ~(np.abs(got - want) <= tol)
    assert not bad.any(), (np.flatnonzero(bad)[:5], got[bad][:5], want[bad][:5])
    assert nrm == pytest.approx(np.linalg.norm(want), rel=1e-13)
    # no less accurate than the FP64 chain of the drop-in evaluation
    op.eval(gpu.from_numpy(u), out64)
    assert np.abs(got - want).max() <= np.abs(out64.numpy() - want).max() + tol.max()


def test_mixed_solve_agrees_with_fp64(gpu):
    G = _G()
    n = 31
    op = G.Bratu3D(gpu, n, 6.0)
    pc64 = G.Provider.poisson_mg(gpu, n)
    pc32 = G.Provider.poisson_mg(gpu, n, precision=G.FP32)
    x64, x32 = gpu.vec(n ** 3), gpu.vec(n ** 3)
    r64 = G.newton_krylov(op, x64, G.default_params(rtol_nl=1e-10, gmres_restart=30), pc64)
    r32 = G.newton_krylov(op, x32, G.default_params(rtol_nl=1e-10, gmres_restart=30, flexible=1,
                                                    jvp_precision=G.FP32), pc32)
    assert r64["converged"] and r32["converged"]
    assert r32["res"] <= 1e-10 * r32["res0"]
    a, b = x32.numpy(), x64.numpy()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-8


@pytest.mark.parametrize("lam", [3.1, 6.0])
def test_tight_products_save_a_newton_step(gpu, lam):
    """With the Jacobian-aware coarse levels, FP32 products leave the last linear solves short of the
    accuracy the quadratic Newton step needs (FP32 arithmetic on the Laplacian of a smooth vector
    loses digits to cancellation); taking those products to FP64 accuracy (jvp_tight) converges
    in fewer Newton steps and linear iterations, to the same solution (1e-8 of the FP64 drop-in's)."""
    G = _G()
    n = 127
    op = G.Bratu3D(gpu, n, lam)
    p = G.default_params(rtol_nl=1e-10, gmres_restart=30, flexible=1, jvp_precision=G.FP32, orth=G.CGS1)
    pt = G.default_params(rtol_nl=1e-10, gmres_restart=30, flexible=1, jvp_precision=G.FP32, orth=G.CGS1,
                          jvp_tight=1)
    pcj = G.Provider.jacobian_mg(gpu, n)
    x64, xf, xt = gpu.vec(n ** 3), gpu.vec(n ** 3), gpu.vec(n ** 3)
    G.newton_krylov(op, x64, G.default_params(rtol_nl=1e-10, gmres_restart=30), G.Provider.poisson_mg(gpu, n))
    rf = G.newton_krylov(op, xf, p, pcj)
    rt = G.newton_krylov(op, xt, pt, pcj)
    assert rf["converged"] and rt["converged"]
    assert rt["res"] <= 1e-10 * rt["res0"]
    assert rel_err(xt.numpy(), x64.numpy()) < 1e-8
    assert rt["iters"] <= rf["iters"] and rt["n_lin_iters"] <= rf["n_lin_iters"], (rt, rf)
    if lam == 6.0:  # the benchmark's lambda: 4 Newton steps and 9 linear iterations against 5 and 11
        assert rt["iters"] < rf["iters"] and rt["n_lin_iters"] < rf["n_lin_iters"], (rt, rf)
    # the host entry with the same preconditioner and parameters gives the same solve
    xh, rh = G.solve_bratu3d_host(gpu, n, lam, np.zeros(n ** 3), method="nk", precond="jacobian_mg",
                                  mg_precision=G.FP32, params=pt)
    assert rh["iters"] == rt["iters"] and rh["n_lin_iters"] == rt["n_lin_iters"]
    assert np.array_equal(xh, xt.numpy())


@pytest.mark.parametrize("lam", [2.5, 4.7, 6.3])
def test_jacobian_aware_coarse_levels_save_iterations(gpu, lam):
    """The FP32 V-cycle whose coarse levels (n <= 15) solve with the Jacobian -Lap_h - lambda e^u
    instead of -Lap_h: inside the mixed FGMRES it reaches the same 1e-10 solution (within 1e-8 of the
    FP64 drop-in's) with fewer linear iterations than the Poisson V-cycle, and no more Newton steps,
    at lambda values away from the benchmark's."""
    G = _G()
    n = 63
    op = G.Bratu3D(gpu, n, lam)
    p = G.default_params(rtol_nl=1e-10, gmres_restart=30, flexible=1, jvp_precision=G.FP32, orth=G.CGS1)
    x64, xp, xj = gpu.vec(n ** 3), gpu.vec(n ** 3), gpu.vec(n ** 3)
    G.newton_krylov(op, x64, G.default_params(rtol_nl=1e-10, gmres_restart=30), G.Provider.poisson_mg(gpu, n))
    rp = G.newton_krylov(op, xp, p, G.Provider.poisson_mg(gpu, n, precision=G.FP32))
    rj = G.newton_krylov(op, xj, p, G.Provider.jacobian_mg(gpu, n))
    assert rp["converged"] and rj["converged"]
    assert rj["res"] <= 1e-10 * rj["res0"]
    assert rel_err(xj.numpy(), x64.numpy()) < 1e-8
    assert rj["iters"] <= rp["iters"]
    assert rj["n_lin_iters"] < rp["n_lin_iters"], (rj, rp)


@pytest.mark.parametrize("n,lam,start", [(2, 6.0, "zero"), (7, 6.0, "zero"), (16, 6.0, "zero"), (33, 9.0, "zero"),
                                         (31, 6.0, "profile"), (31, 0.0, "zero")])
def test_benchmark_mixed_path_sizes_lambdas_starts(gpu, n, lam, start):
    """The benchmark's mixed path (FGMRES(30) with one-pass classical Gram-Schmidt, the FP32 V-cycle with
    Jacobian-aware coarse levels, FP32 products and, in the tight linear solves, products of FP64
    accuracy) away from the benchmark's grid: a hierarchy of one level (n = 2, 16), an odd chain ending
    in 1 (7, 31), an even coarsest level (33 -> 16), near the fold (lambda = 9), a nonzero start, and
    lambda = 0 from u0 = 0, where F(u0) = 0 and both paths stop before a step.  Grids without an odd
    chain down to n <= 15 have no Jacobian-aware levels (NOT_SUPPORTED) and take the FP32 Poisson
    V-cycle.  It reaches the FP64 drop-in's solution to 1e-8."""
    G = _G()
    N = n ** 3
    op = G.Bratu3D(gpu, n, lam)
    pm = G.default_params(rtol_nl=1e-10, gmres_restart=30, flexible=1, jvp_precision=G.FP32, orth=G.CGS1,
                          jvp_tight=1)
    x64, xm = gpu.vec(N), gpu.vec(N)
    if start == "profile":
        i, j, k = np.indices((n, n, n)) + 1.0
        u0 = (0.3 * np.sin(np.pi * i / (n + 1)) * np.sin(np.pi * j / (n + 1)) * np.sin(np.pi * k / (n + 1))).ravel()
        x64.copy_from(gpu.from_numpy(u0))
        xm.copy_from(gpu.from_numpy(u0))
    try:
        pc = G.Provider.jacobian_mg(gpu, n)
    except G.NumaGPUError as e:  # no odd chain of levels down to n <= 15: the FP32 Poisson V-cycle instead
        assert e.code == NOT_SUPPORTED and n in (2, 16, 33), (n, str(e))
        pc = G.Provider.poisson_mg(gpu, n, precision=G.FP32)
    r64 = G.newton_krylov(op, x64, G.default_params(rtol_nl=1e-10, gmres_restart=30), G.Provider.poisson_mg(gpu, n))
    rm = G.newton_krylov(op, xm, pm, pc)
    assert r64["converged"] and rm["converged"], (r64, rm)
    if lam == 0.0:
        assert rm["iters"] == 0 and r64["iters"] == 0
        assert not xm.numpy().any() and not x64.numpy().any()
        return
    assert rm["res"] <= 1e-10 * rm["res0"]
    assert rel_err(xm.numpy(), x64.numpy()) < 1e-8, (rel_err(xm.numpy(), x64.numpy()), r64, rm)
