"""The learned preconditioner's tensor-core kernels against the CPU restatement
(oracle/learned_oracle.py): the 3x3x3 convolution (tcgen05, BF16 operands, FP32 accumulation) and
its adjoint.  Inputs are rounded to BF16 on both sides, so the only difference left is the order of
the FP32 accumulation: relative error well below 1e-5."""
from __future__ import annotations

import numpy as np
import pytest

from oracle.learned_oracle import bf16, conv3d, conv3d_adjoint, conv3d_wgrad

pytestmark = pytest.mark.gpu


def _G():
    import numa_gpu
    return numa_gpu


@pytest.mark.parametrize("n", [1, 3, 7, 15, 31])
@pytest.mark.parametrize("cin,cout", [(16, 16), (16, 32), (32, 16), (32, 32)])
def test_conv3d_tensor_cores(gpu, n, cin, cout):
    G = _G()
    rng = np.random.default_rng(7 * n + cin + 3 * cout)
    x = bf16(rng.standard_normal((n ** 3, cin)))
    w = bf16(rng.standard_normal((27, cin, cout)) * 0.2)
    b = rng.standard_normal(cout).astype(np.float32)
    y = G.diag_conv3d(gpu, n, x, w, b)
    ref = conv3d(x, w, n, b)
    scale = np.abs(ref).max() + 1e-30
    assert np.abs(y - ref).max() / scale < 1e-5


@pytest.mark.parametrize("n", [3, 15])
@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 16)])
def test_conv3d_adjoint_tensor_cores(gpu, n, cin, cout):
    G = _G()
    rng = np.random.default_rng(11 * n + cin)
    g = bf16(rng.standard_normal((n ** 3, cout)))
    w = bf16(rng.standard_normal((27, cin, cout)) * 0.2)
    dx = G.diag_conv3d(gpu, n, g, w, adjoint=True)
    ref = conv3d_adjoint(g, w, n)
    assert np.abs(dx - ref).max() / (np.abs(ref).max() + 1e-30) < 1e-5


@pytest.mark.parametrize("n", [1, 3, 7, 15, 31, 63])
@pytest.mark.parametrize("cin,cout", [(16, 16), (16, 32), (32, 16), (32, 32)])
def test_conv3d_weight_gradient_tensor_cores(gpu, n, cin, cout):
    """The weight gradient as implicit GEMMs on the tensor cores (MN-major operands straight from the
    plane layout, the three dz taps stacked along M) against the FP64 sums of the oracle on the same
    BF16 inputs; the bias gradient beside it."""
    if n == 63 and (cin, cout) != (32, 32):
        pytest.skip("63^3 once, at the largest channel counts")
    G = _G()
    rng = np.random.default_rng(13 * n + cin + 5 * cout)
    x = bf16(rng.standard_normal((n ** 3, cin)))
    g = bf16(rng.standard_normal((n ** 3, cout)))
    dw, db = G.diag_conv3d_wgrad(gpu, n, x, g)
    ref_w, ref_b = conv3d_wgrad(x, g, n)
    assert np.abs(dw - ref_w).max() / (np.abs(ref_w).max() + 1e-30) < 1e-5
    assert np.abs(db - ref_b).max() / (np.abs(ref_b).max() + 1e-30) < 1e-5


def test_network_forward_and_gradient(gpu):
    """The whole network, forward and backward, on the GPU against the oracle in its BF16 mode (every
    stored activation and gradient rounded as the GPU does): outputs, loss and each layer's weight
    gradient agree to the FP32-accumulation level, up to the odd BF16 value rounded the other way."""
    from oracle.learned_oracle import LAYERS, unet_backward, unet_forward
    G = _G()
    n0 = 15
    net = G.LearnedNet(gpu, n0, seed=5)
    p = net.get_params()
    rng = np.random.default_rng(9)
    feat = rng.standard_normal((n0 ** 3, 3)).astype(np.float32)
    t = (rng.standard_normal(n0 ** 3) * 0.1).astype(np.float32)
    out = net.forward(feat)
    ref, cache = unet_forward(p, feat, n0, bf=True)
    assert np.linalg.norm(out - ref) <= 1e-2 * np.linalg.norm(ref)
    loss, g = net.gradient(feat, t)
    rloss, rg = unet_backward(cache, t, bf=True)
    assert abs(loss - rloss) <= 1e-3 * rloss
    o, errs = 0, []
    for ci, co, _, _ in LAYERS:
        sz = 27 * ci * co + co
        a, b = g[o:o + sz], rg[o:o + sz]
        errs.append(float(np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30)))
        o += sz
    cos = float(g @ rg) / (np.linalg.norm(g) * np.linalg.norm(rg))
    print("per-layer relative gradient error", ["%.2e" % e for e in errs], "cosine", cos)
    assert max(errs) <= 5e-2, errs
    assert cos > 0.999


def _solve(G, gpu, n, lam, provider, params):
    op = G.Bratu3D(gpu, n, lam)
    x = gpu.vec(n ** 3)
    r = G.newton_krylov(op, x, params, provider)
    return x.numpy(), r


def test_learned_preconditioner_trains_and_solves(gpu):
    """Training on the GPU lowers the loss; inside FGMRES the learned preconditioner reaches the
    same solution as the plain FP64 path on a held-out lambda (what it gains in iterations is
    printed: the test asserts convergence and the solution, not a gain)."""
    G = _G()
    n, n0 = 31, 15
    net = G.LearnedNet(gpu, n0, seed=3)
    rep = net.train(n, instances=4, states=3, rhs_per_state=2, krylov_per_state=8, epochs=8, batch=4, lr=2e-3,
                    seed=11)
    print("training", rep)
    assert rep["samples"] == 4 * 3 * 11
    assert rep["loss_last"] < 0.1 * rep["target_ms"]  # well below predicting zero
    assert rep["loss_last"] < rep["loss_first"]
    lam = 5.77  # not a training draw
    fp = G.default_params(rtol_nl=1e-10, gmres_restart=30)
    x64, r64 = _solve(G, gpu, n, lam, G.Provider.poisson_mg(gpu, n), fp)
    mp = G.default_params(rtol_nl=1e-10, gmres_restart=30, flexible=1, jvp_precision=G.FP32)
    xm, rm = _solve(G, gpu, n, lam, G.Provider.poisson_mg(gpu, n, precision=G.FP32), mp)
    pl = G.Provider.learned(gpu, n, net, stall=0.9)
    xl, rl = _solve(G, gpu, n, lam, pl, mp)
    applies, fallbacks = pl.learned_stats()
    print("plain", r64["iters"], r64["n_lin_iters"], "mixed", rm["iters"], rm["n_lin_iters"], "learned", rl["iters"],
          rl["n_lin_iters"], "net applies", applies, "fallbacks", fallbacks)
    assert rl["converged"] == 1 and applies > 0
    assert np.linalg.norm(xl - x64) <= 1e-8 * np.linalg.norm(x64)


def test_training_is_repeatable(gpu):
    """The same seeds give the same training data and the same network, bit for bit, run after run in
    one process (the data come from solves whose kernels and reductions have a fixed order)."""
    G = _G()
    runs = []
    for _ in range(2):
        net = G.LearnedNet(gpu, 15, seed=3)
        rep = net.train(31, instances=2, states=2, rhs_per_state=1, krylov_per_state=4, epochs=2, batch=4, lr=2e-3,
                        seed=11)
        runs.append((rep["target_ms"], rep["loss_first"], net.get_params()))
    assert runs[0][0] == runs[1][0]
    assert np.array_equal(runs[0][2], runs[1][2])


def test_stagnation_falls_back_to_the_vcycle(gpu):
    """A network that corrects in the wrong direction (an untrained one with its weights scaled
    up tenfold) makes an FGMRES iteration stall; the provider then hands the rest of that linear
    solve to the plain V-cycle, and the Newton solve still converges to the FP64 path's solution."""
    G = _G()
    n, n0 = 31, 15
    net = G.LearnedNet(gpu, n0, seed=3)
    net.set_params(net.get_params() * 10.0)
    mp = G.default_params(rtol_nl=1e-10, gmres_restart=30, flexible=1, jvp_precision=G.FP32)
    pl = G.Provider.learned(gpu, n, net, stall=0.9)
    xl, rl = _solve(G, gpu, n, 4.2, pl, mp)
    applies, fallbacks = pl.learned_stats()
    x64, _ = _solve(G, gpu, n, 4.2, G.Provider.poisson_mg(gpu, n), G.default_params(rtol_nl=1e-10, gmres_restart=30))
    assert fallbacks > 0, (applies, fallbacks)
    assert rl["converged"] == 1 and rl["res"] <= 1e-10 * rl["res0"]
    assert np.linalg.norm(xl - x64) <= 1e-8 * np.linalg.norm(x64)
