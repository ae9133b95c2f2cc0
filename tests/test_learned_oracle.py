"""The learned preconditioner's CPU restatement checked against itself: the adjoint convolution is
the transpose of the convolution (<conv(x), g> = <x, conv_adjoint(g)>), and BF16 rounding is
round-to-nearest-even."""
from __future__ import annotations

import numpy as np

from oracle.learned_oracle import bf16, conv3d, conv3d_adjoint


def test_adjoint_identity():
    rng = np.random.default_rng(0)
    n, cin, cout = 5, 3, 4
    x = rng.standard_normal((n ** 3, cin))
    g = rng.standard_normal((n ** 3, cout))
    w = rng.standard_normal((27, cin, cout))
    lhs = float(np.sum(conv3d(x, w, n) * g))
    rhs = float(np.sum(x * conv3d_adjoint(g, w, n)))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.0078125, 1.005859375, 3.0e38, -2.5], dtype=np.float32)
    r = bf16(v)
    assert r[0] == 1.0 and r[2] == 1.0078125
    assert r[1] == 1.0  # a tie goes to the even neighbour
    assert r[3] == 1.0078125
    assert r[5] == -2.5


def test_transfer_adjoints():
    from oracle.learned_oracle import prolong, restrict
    rng = np.random.default_rng(1)
    nf, nc = 7, 3
    f = rng.standard_normal((nf ** 3, 2))
    c = rng.standard_normal((nc ** 3, 2))
    # <R f, c> = <f, P c / 8>
    assert abs(np.sum(restrict(f, nf) * c) - np.sum(f * prolong(c, nc)) / 8.0) < 1e-12


def test_network_gradient_finite_differences():
    """The oracle's backward pass (exact arithmetic, no BF16) against central differences of its
    own loss along a random direction in each layer's parameters.  The step is small (1e-7) so that
    no ReLU changes side within it."""
    from oracle.learned_oracle import LAYERS, num_params, unet_backward, unet_forward
    rng = np.random.default_rng(2)
    n0 = 15
    p = rng.standard_normal(num_params()) * 0.05
    feat = rng.standard_normal((n0 ** 3, 3))
    t = rng.standard_normal(n0 ** 3) * 0.1

    def loss_of(q):
        out, _ = unet_forward(q, feat, n0, bf=False)
        return float(np.mean((out - t) ** 2))

    _, cache = unet_forward(p, feat, n0, bf=False)
    _, g = unet_backward(cache, t, bf=False)
    o = 0
    for ci, co, _, _ in LAYERS:
        sz = 27 * ci * co + co
        d = np.zeros(p.size)
        d[o:o + sz] = rng.standard_normal(sz)
        eps = 1e-7
        fd = (loss_of(p + eps * d) - loss_of(p - eps * d)) / (2 * eps)
        assert abs(fd - float(g @ d)) <= 1e-6 * abs(fd) + 1e-12, (o, fd, float(g @ d))
        o += sz
