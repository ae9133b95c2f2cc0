"""An upper bound on what a coarse-level learned correction can gain (test infrastructure: the CPU
oracle's V-cycle and Jacobian products, numpy for the rest).

The learned preconditioner adds to the Poisson V-cycle a correction that a network computes on the
level of size nc from the residual the V-cycle leaves and the Jacobian coefficient c = lambda e^u:
    z = V(r) + P_nc N(R_nc (r - J V(r)), R_nc c).
No network can do better on that level than the exact coarse solve of the error equation,
N(q, c) = (-Lap_nc - diag(R_nc c))^-1 q, so the Newton-Krylov solve preconditioned with that exact
correction bounds the iterations any trained network of that form could save.  This script counts
them: FGMRES(30) (modified Gram-Schmidt) inside the reference's Newton-Krylov loop (Eisenstat-Walker
forcing, Armijo backtracking, rtol 1e-10), with the plain V-cycle and with the exact correction on each
coarse level given.

    python oracle/learned_bound.py 255 6.0 63,31,15
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
from oracle.oracle_lib import Oracle, default_params  # noqa: E402


def laplacian(m: int) -> sp.csr_matrix:
    """-Lap_h on the m^3 interior grid, h = 1/(m+1), Dirichlet zeros (the 7-point stencil)."""
    h2 = (m + 1.0) ** 2
    e = np.ones(m)
    T = sp.diags([-e[:-1], 2 * e, -e[:-1]], [-1, 0, 1])
    I = sp.identity(m)
    return (h2 * (sp.kron(sp.kron(T, I), I) + sp.kron(sp.kron(I, T), I) + sp.kron(sp.kron(I, I), T))).tocsr()


def fgmres(A, M, b, rtol, m=30, maxit=500):
    """Right-preconditioned flexible GMRES(m) with modified Gram-Schmidt; returns (x, iterations)."""
    bn = np.linalg.norm(b)
    x = np.zeros_like(b)
    it = 0
    r, beta = b.copy(), bn
    while it < maxit:
        V, Z = [r / beta], []
        H = np.zeros((m + 1, m))
        g = np.zeros(m + 1)
        g[0] = beta
        res = beta
        for j in range(m):
            z = M(V[j])
            Z.append(z)
            w = A(z)
            for i in range(j + 1):
                H[i, j] = w @ V[i]
                w = w - H[i, j] * V[i]
            H[j + 1, j] = np.linalg.norm(w)
            V.append(w / H[j + 1, j])
            it += 1
            y, *_ = np.linalg.lstsq(H[:j + 2, :j + 1], g[:j + 2], rcond=None)
            res = np.linalg.norm(g[:j + 2] - H[:j + 2, :j + 1] @ y)
            if res <= rtol * bn:
                break
        x = x + np.array(Z).T @ y
        if res <= rtol * bn:
            break
        r = b - A(x)
        beta = np.linalg.norm(r)
    return x, it


def newton_krylov(o: Oracle, n: int, lam: float, nc: int | None):
    """(total linear iterations, per Newton step, Newton steps) with the plain V-cycle (nc None) or
    the V-cycle plus the exact coarse correction on level nc."""
    N = n ** 3
    p = default_params(rtol_nl=1e-10, gmres_restart=30)
    x = np.zeros(N)
    F = o.eval(n, lam, x)
    rn = np.linalg.norm(F)
    r0, rp, ep = rn, rn, p.eta_init
    its = []
    k = 0
    for k in range(50):
        if rn <= 1e-10 * r0:
            break
        eta = o.forcing(p, k, rn, rp, ep, r0)

        def A(v, x=x):
            return o.jvp(n, lam, x, v)

        if nc is None:
            def M(r):
                return o.mg_apply(n, r)
        else:
            c = lam * np.exp(x)
            m = n
            while m > nc:
                c, m = o.mg_restrict(m, c), (m - 1) // 2
            Jc = (laplacian(nc) - sp.diags(c)).tocsc()
            if nc <= 31:
                solve_c = spla.splu(Jc).solve
            else:
                def solve_c(b, Jc=Jc):
                    return spla.cg(Jc, b, rtol=1e-12, maxiter=5000)[0]

            def M(r):
                z = o.mg_apply(n, r)
                q = r - A(z)
                m = n
                while m > nc:
                    q, m = o.mg_restrict(m, q), (m - 1) // 2
                e = solve_c(q)
                while m < n:
                    e, m = o.mg_prolong_add(m, e, np.zeros((2 * m + 1) ** 3)), 2 * m + 1
                return z + e
        z, it = fgmres(A, M, F, eta)
        its.append(it)
        al = 1.0
        while al >= 1e-4:
            xn = x - al * z
            Fn = o.eval(n, lam, xn)
            if np.linalg.norm(Fn) <= (1 - 1e-4 * al) * rn:
                break
            al *= 0.5
        x, F = xn, Fn
        rp, rn, ep = rn, np.linalg.norm(F), eta
    return sum(its), its, k


def main(argv):
    n = int(argv[1]) if len(argv) > 1 else 63
    lam = float(argv[2]) if len(argv) > 2 else 6.0
    levels = [int(a) for a in argv[3].split(",")] if len(argv) > 3 else [15, 7]
    o = Oracle()
    print("plain V-cycle", newton_krylov(o, n, lam, None), flush=True)
    for nc in levels:
        print("exact coarse correction on", nc, newton_krylov(o, n, lam, nc), flush=True)


if __name__ == "__main__":
    main(sys.argv)
