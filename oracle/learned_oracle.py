"""CPU restatement of the learned preconditioner's arithmetic: test infrastructure only (the
checker for the GPU's tensor-core convolutions, transfers and the network's forward and
backward passes).  numpy, FP64 accumulation; BF16 rounding (round to nearest even) wherever the
GPU stores a BF16 value, so the comparison isolates the FP32 accumulation order."""
from __future__ import annotations

import numpy as np


def bf16(a) -> np.ndarray:
    """Round float32 values to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def taps():
    """(tap index, dz, dy, dx) with tap = (dz*3 + dy)*3 + dx and offsets d - 1."""
    for t in range(27):
        yield t, t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1


def conv3d(x: np.ndarray, w: np.ndarray, n: int, bias=None) -> np.ndarray:
    """y[v][co] = bias[co] + sum_{tap, ci} x[v + tap][ci] w[tap][ci][co], zero outside the grid.
    x: [n^3, cin] (z, y, x order, x fastest); w: [27, cin, cout]; FP64 accumulation."""
    cin, cout = w.shape[1], w.shape[2]
    xp = np.zeros((n + 2, n + 2, n + 2, cin))
    xp[1:-1, 1:-1, 1:-1] = np.asarray(x, dtype=np.float64).reshape(n, n, n, cin)
    y = np.zeros((n, n, n, cout))
    for t, dz, dy, dx in taps():
        y += xp[1 + dz:n + 1 + dz, 1 + dy:n + 1 + dy, 1 + dx:n + 1 + dx] @ np.asarray(w[t], dtype=np.float64)
    if bias is not None:
        y += np.asarray(bias, dtype=np.float64)
    return y.reshape(n ** 3, cout)


def conv3d_adjoint(g: np.ndarray, w: np.ndarray, n: int) -> np.ndarray:
    """The gradient of conv3d with respect to x: dx[u][ci] = sum_{tap, co} g[u - tap][co] w[tap][ci][co]."""
    wf = np.stack([np.asarray(w[26 - t], dtype=np.float64).T for t in range(27)])  # [27][cout][cin]
    return conv3d(g, wf, n)


def conv3d_wgrad(x: np.ndarray, g: np.ndarray, n: int):
    """The gradients of conv3d with respect to its weights and bias: dw[tap][ci][co] =
    sum_v x[v + tap][ci] g[v][co] (x zero outside the grid), db[co] = sum_v g[v][co]; FP64."""
    ci, co = x.shape[1], g.shape[1]
    xp = np.zeros((n + 2, n + 2, n + 2, ci))
    xp[1:-1, 1:-1, 1:-1] = np.asarray(x, dtype=np.float64).reshape(n, n, n, ci)
    gg = np.asarray(g, dtype=np.float64).reshape(-1, co)
    gw = np.zeros((27, ci, co))
    for t, dz, dy, dx in taps():
        gw[t] = xp[1 + dz:n + 1 + dz, 1 + dy:n + 1 + dy, 1 + dx:n + 1 + dx].reshape(-1, ci).T @ gg
    return gw, gg.sum(axis=0)


# ------------------------------------------------------------------------------ the network
# (cin, cout, level, relu) of e0a e0b e1a e1b e2a e2b e3a e3b d2 d1 d0a d0b — the layer table of
# the GPU network (chebyshev-nonlinear-lab_gb300/csrc/learned_net.cu).
LAYERS = [(16, 16, 0, True), (16, 16, 0, True), (16, 32, 1, True), (32, 32, 1, True), (32, 32, 2, True),
          (32, 32, 2, True), (32, 32, 3, True), (32, 32, 3, True), (32, 32, 2, True), (32, 16, 1, True),
          (16, 16, 0, True), (16, 16, 0, False)]
E0A, E0B, E1A, E1B, E2A, E2B, E3A, E3B, D2, D1, D0A, D0B = range(12)


def num_params() -> int:
    return sum(27 * ci * co + co for ci, co, _, _ in LAYERS)


def split_params(p: np.ndarray):
    """[(W [27, cin, cout], b [cout])] in layer order from the flat FP32 parameter vector."""
    out, o = [], 0
    for ci, co, _, _ in LAYERS:
        w = p[o:o + 27 * ci * co].reshape(27, ci, co)
        o += 27 * ci * co
        b = p[o:o + co]
        o += co
        out.append((w, b))
    return out


def flat_grads(gs) -> np.ndarray:
    return np.concatenate([np.concatenate([gw.ravel(), gb.ravel()]) for gw, gb in gs])


def restrict(x: np.ndarray, n: int) -> np.ndarray:
    """Full weighting per channel, fine n^3 (odd) -> coarse ((n-1)/2)^3; x [n^3, C]."""
    nc = (n - 1) // 2
    C = x.shape[1]
    f = np.asarray(x, dtype=np.float64).reshape(n, n, n, C)
    w = (0.25, 0.5, 0.25)
    out = np.zeros((nc, nc, nc, C))
    for a in range(3):
        for b in range(3):
            for c in range(3):
                out += w[a] * w[b] * w[c] * f[a:a + 2 * nc:2, b:b + 2 * nc:2, c:c + 2 * nc:2]
    return out.reshape(nc ** 3, C)


def _interp_matrix(nf: int, nc: int) -> np.ndarray:
    m = np.zeros((nf, nc))
    for f in range(nf):
        if f & 1:
            m[f, (f - 1) // 2] = 1.0
        else:
            r = f // 2
            if r >= 1:
                m[f, r - 1] = 0.5
            if r < nc:
                m[f, r] = 0.5
    return m


def prolong(x: np.ndarray, nc: int) -> np.ndarray:
    """Trilinear interpolation per channel, coarse nc^3 -> fine (2 nc + 1)^3; x [nc^3, C]."""
    nf = 2 * nc + 1
    C = x.shape[1]
    m = _interp_matrix(nf, nc)
    c = np.asarray(x, dtype=np.float64).reshape(nc, nc, nc, C)
    return np.einsum("ai,bj,ck,ijkq->abcq", m, m, m, c).reshape(nf ** 3, C)


def _r(a, bf):
    return bf16(a).astype(np.float64) if bf else np.asarray(a, dtype=np.float64)


def unet_forward(params: np.ndarray, feat: np.ndarray, n0: int, bf: bool = True):
    """Output [n0^3] (channel 0 of d0b) and the activations, from features [n0^3, 3]; bf: round
    every stored activation and the weights to BF16 as the GPU does."""
    ps = split_params(np.asarray(params, dtype=np.float32 if bf else np.float64))
    W = [(_r(w, bf), np.asarray(b, dtype=np.float64)) for w, b in ps]
    ns = [n0, (n0 - 1) // 2, (n0 - 3) // 4, (n0 - 7) // 8]
    N0 = n0 ** 3
    x = np.zeros((N0, 16))
    x[:, :3] = feat
    x = _r(x, bf)
    A = {"in": x}

    def conv(l, inp):
        ci, co, lv, relu = LAYERS[l]
        y = conv3d(inp, W[l][0], ns[lv], W[l][1])
        if relu:
            y = np.maximum(y, 0.0)
        return y

    A["e0a"] = _r(conv(E0A, A["in"]), bf)
    A["s0"] = _r(conv(E0B, A["e0a"]), bf)
    A["r1"] = _r(restrict(A["s0"], ns[0]), bf)
    A["e1a"] = _r(conv(E1A, A["r1"]), bf)
    A["s1"] = _r(conv(E1B, A["e1a"]), bf)
    A["r2"] = _r(restrict(A["s1"], ns[1]), bf)
    A["e2a"] = _r(conv(E2A, A["r2"]), bf)
    A["s2"] = _r(conv(E2B, A["e2a"]), bf)
    A["r3"] = _r(restrict(A["s2"], ns[2]), bf)
    A["e3a"] = _r(conv(E3A, A["r3"]), bf)
    A["e3b"] = _r(conv(E3B, A["e3a"]), bf)
    A["u2"] = _r(A["s2"] + prolong(A["e3b"], ns[3]), bf)
    A["d2"] = _r(conv(D2, A["u2"]), bf)
    A["u1"] = _r(A["s1"] + prolong(A["d2"], ns[2]), bf)
    A["d1"] = _r(conv(D1, A["u1"]), bf)
    A["u0"] = _r(A["s0"] + prolong(A["d1"], ns[1]), bf)
    A["d0a"] = _r(conv(D0A, A["u0"]), bf)
    out = conv(D0B, A["d0a"])
    A["out"] = out
    return out[:, 0], (A, W, ns)


def unet_backward(cache, target: np.ndarray, bf: bool = True):
    """Loss mean (out - t)^2 and its gradient (flat, parameter order) by the adjoint steps of the
    GPU's backward pass (BF16 rounding of every stored gradient when bf)."""
    A, W, ns = cache
    N0 = ns[0] ** 3
    d = A["out"][:, 0] - target
    loss = float(np.mean(d * d))
    G = [None] * 12

    def dw(l, x, g):
        ci, co, lv, _ = LAYERS[l]
        n = ns[lv]
        xp = np.zeros((n + 2, n + 2, n + 2, ci))
        xp[1:-1, 1:-1, 1:-1] = x.reshape(n, n, n, ci)
        gg = g.reshape(n, n, n, co)
        gw = np.zeros((27, ci, co))
        for t, dz, dy, dx in taps():
            xs = xp[1 + dz:n + 1 + dz, 1 + dy:n + 1 + dy, 1 + dx:n + 1 + dx].reshape(-1, ci)
            gw[t] = xs.T @ gg.reshape(-1, co)
        G[l] = (gw, g.sum(axis=0))

    def adj(l, g):
        ci, co, lv, _ = LAYERS[l]
        return _r(conv3d_adjoint(g, W[l][0], ns[lv]), bf)

    g_out = np.zeros((N0, 16))
    g_out[:, 0] = 2.0 * d / N0
    g_out = _r(g_out, bf)
    def mask(g, y, l):  # through layer l's ReLU (whose output is y)
        return np.where(y > 0, g, 0.0) if LAYERS[l][3] else g

    dw(D0B, A["d0a"], g_out)
    g = mask(adj(D0B, g_out), A["d0a"], D0A)
    dw(D0A, A["u0"], g)
    g_u0 = adj(D0A, g)
    g = mask(_r(8.0 * restrict(g_u0, ns[0]), bf), A["d1"], D1)
    dw(D1, A["u1"], g)
    g_u1 = adj(D1, g)
    g = mask(_r(8.0 * restrict(g_u1, ns[1]), bf), A["d2"], D2)
    dw(D2, A["u2"], g)
    g_u2 = adj(D2, g)
    g = mask(_r(8.0 * restrict(g_u2, ns[2]), bf), A["e3b"], E3B)
    dw(E3B, A["e3a"], g)
    g = mask(adj(E3B, g), A["e3a"], E3A)
    dw(E3A, A["r3"], g)
    g_r3 = adj(E3A, g)
    g_u2 = mask(_r(g_u2 + 0.125 * prolong(g_r3, ns[3]), bf), A["s2"], E2B)
    dw(E2B, A["e2a"], g_u2)
    g = mask(adj(E2B, g_u2), A["e2a"], E2A)
    dw(E2A, A["r2"], g)
    g_r2 = adj(E2A, g)
    g_u1 = mask(_r(g_u1 + 0.125 * prolong(g_r2, ns[2]), bf), A["s1"], E1B)
    dw(E1B, A["e1a"], g_u1)
    g = mask(adj(E1B, g_u1), A["e1a"], E1A)
    dw(E1A, A["r1"], g)
    g_r1 = adj(E1A, g)
    g_u0 = mask(_r(g_u0 + 0.125 * prolong(g_r1, ns[1]), bf), A["s0"], E0B)
    dw(E0B, A["e0a"], g_u0)
    g = mask(adj(E0B, g_u0), A["e0a"], E0A)
    dw(E0A, A["in"], g)
    return loss, flat_grads(G)
