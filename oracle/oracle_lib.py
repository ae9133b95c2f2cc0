"""ctypes front end of the oracle libraries (test infrastructure only).

``Oracle()`` loads oracle/_build/liboracle.so (the CPU restatement, built on demand);
``Oracle.reference()`` loads oracle/_ref/libnuma_ref.so (the reference's own headers compiled
here) when it exists.  Both export the same C signatures under the prefixes ``oracle_`` and
``ref_``.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

F64P = C.POINTER(C.c_double)


class KrylovParams(C.Structure):
    """numa_krylov_params of include/numa_gpu.h."""
    _fields_ = [
        ("rtol_nl", C.c_double), ("max_nl", C.c_uint64), ("eta_init", C.c_double),
        ("eta_max", C.c_double), ("gamma", C.c_double), ("alpha", C.c_double),
        ("eta2_factor", C.c_double), ("eta2_max", C.c_double), ("gmres_restart", C.c_uint64),
        ("gmres_max_iters", C.c_uint64), ("armijo", C.c_double), ("min_lambda", C.c_double),
        ("recycle", C.c_int32), ("jvp_mode", C.c_int32), ("d2_mode", C.c_int32),
        ("orth", C.c_int32), ("flexible", C.c_int32), ("jvp_precision", C.c_int32),
        ("jvp_tight", C.c_int32), ("coarse_jacobian", C.c_int32), ("reserved", C.c_int32 * 2),
    ]


class KrylovResult(C.Structure):
    """numa_krylov_result of include/numa_gpu.h."""
    _fields_ = [
        ("converged", C.c_int32), ("status", C.c_int32), ("iters", C.c_uint64),
        ("n_F", C.c_uint64), ("n_JVP", C.c_uint64), ("n_D2", C.c_uint64),
        ("n_lin_iters", C.c_uint64), ("n_lin_failures", C.c_uint64), ("n_prec", C.c_uint64),
        ("res0", C.c_double), ("res", C.c_double), ("t_F", C.c_double), ("t_JVP", C.c_double),
        ("t_D2", C.c_double), ("t_prec", C.c_double), ("t_setup_dynamic", C.c_double),
        ("t_total", C.c_double),
    ]


class GmresResult(C.Structure):
    """numa_gmres_result of include/numa_gpu.h."""
    _fields_ = [
        ("iters", C.c_uint64), ("matvecs", C.c_uint64), ("precs", C.c_uint64),
        ("rel_res", C.c_double), ("converged", C.c_int32), ("breakdown", C.c_int32),
    ]


def default_params(**kw) -> KrylovParams:
    """KrylovParams{} defaults (methods/krylov_newton.hpp:24-38), overridden by keywords."""
    p = KrylovParams()
    p.rtol_nl, p.max_nl, p.eta_init, p.eta_max = 1e-8, 50, 0.5, 0.9
    p.gamma, p.alpha, p.eta2_factor, p.eta2_max = 0.9, 2.0, 10.0, 0.5
    p.gmres_restart, p.gmres_max_iters, p.armijo, p.min_lambda = 50, 500, 1e-4, 1e-4
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def struct_dict(s) -> dict:
    return {name: getattr(s, name) for name, _ in s._fields_ if name != "reserved"}


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(F64P)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def make_point(N: int, scale: float) -> np.ndarray:
    """The reference tests' deterministic vector s*sin(0.37 i + 0.5) (tests/test_operators.cpp:19-23)."""
    return scale * np.sin(0.37 * np.arange(N, dtype=np.float64) + 0.5)


METHODS = {"nk": 0, "cheb": 1, "rec": 2, "tf2018": 3}
PRECONDS = {"none": 0, "mg": 1, "jacobi": 2}


class Oracle:
    def __init__(self, path: str | Path | None = None, prefix: str = "oracle_"):
        if path is None:
            from .build import build_oracle
            path = build_oracle()
        self.path = Path(path)
        self.lib = C.CDLL(str(self.path))
        self.prefix = prefix
        L, P = self.lib, prefix
        sz, dbl, i32 = C.c_size_t, C.c_double, C.c_int

        def fn(name, args, res=None):
            f = getattr(L, P + name)
            f.argtypes = args
            f.restype = res
            return f

        self._eval = fn("bratu3d_eval", [sz, dbl, F64P, F64P])
        self._jvp = fn("bratu3d_jvp", [sz, dbl, F64P, F64P, F64P, i32])
        self._d2 = fn("bratu3d_d2", [sz, dbl, F64P, F64P, F64P, i32])
        self._jdiag = fn("bratu3d_jacobi_diag", [sz, dbl, F64P, F64P])
        self._levels = fn("mg_levels", [sz, i32, i32], i32)
        self._mg_apply = fn("mg_apply", [sz, i32, i32, F64P, F64P], i32)
        self._gmres = fn("gmres_bratu3d", [sz, dbl, F64P, i32, i32, F64P, F64P, dbl, sz, sz, i32,
                                           C.POINTER(GmresResult)], i32)
        self._pair = fn("gmres_recycle_pair", [sz, dbl, F64P, i32, F64P, F64P, dbl, sz, sz, F64P,
                                               F64P, C.POINTER(C.c_size_t), C.POINTER(GmresResult),
                                               C.POINTER(GmresResult)], i32)
        self._gpois = fn("gmres_poisson_mg", [sz, F64P, F64P, dbl, sz, sz, C.POINTER(GmresResult)], i32)
        self._solve = fn("solve_bratu3d", [sz, dbl, i32, i32, C.POINTER(KrylovParams), F64P, F64P,
                                           C.POINTER(KrylovResult)], i32)
        self._forcing = fn("forcing", [C.POINTER(KrylovParams), sz, dbl, dbl, dbl, dbl], dbl)
        self._bexact = fn("burgers2d_exact", [sz, dbl, dbl, dbl, F64P], i32)
        self._beval = fn("burgers2d_eval", [sz, dbl, dbl, dbl, F64P, F64P], i32)
        self._bjvp = fn("burgers2d_jvp", [sz, dbl, dbl, dbl, F64P, F64P, F64P, i32], i32)
        self._bd2 = fn("burgers2d_d2", [sz, dbl, dbl, dbl, F64P, F64P, F64P, i32], i32)
        self._hlev = fn("hmg2d_levels", [sz, dbl, dbl], i32)
        self._happly = fn("hmg2d_apply", [sz, dbl, dbl, i32, i32, F64P, F64P], i32)
        self._bsolve = fn("solve_burgers2d", [sz, dbl, dbl, dbl, i32, i32, C.POINTER(KrylovParams), F64P, F64P,
                                              C.POINTER(KrylovResult)], i32)
        self._r1prev = fn("bruss1d_previous", [sz, dbl, F64P], i32)
        self._r1eval = fn("bruss1d_eval", [sz, dbl, F64P, F64P], i32)
        self._r1jvp = fn("bruss1d_jvp", [sz, dbl, F64P, F64P, F64P, i32], i32)
        self._r1d2 = fn("bruss1d_d2", [sz, dbl, F64P, F64P, F64P, i32], i32)
        self._r1jac = fn("bruss1d_jacobi_apply", [sz, dbl, F64P, F64P, F64P], i32)
        self._r1solve = fn("solve_bruss1d", [sz, dbl, i32, i32, C.POINTER(KrylovParams), F64P, F64P,
                                             C.POINTER(KrylovResult)], i32)
        if prefix == "oracle_":
            self._r2eval = fn("bruss2d_eval", [sz, F64P, F64P, F64P, F64P], i32)
            self._r2jvp = fn("bruss2d_jvp", [sz, F64P, F64P, F64P, F64P, F64P, i32], i32)
            self._r2d2 = fn("bruss2d_d2", [sz, F64P, F64P, F64P, F64P, F64P, i32], i32)
            self._bmglev = fn("bmg2d_levels", [sz], i32)
            self._bmgapply = fn("bmg2d_apply", [sz, F64P, F64P, i32, i32, F64P, F64P], i32)
            self._r2solve = fn("solve_bruss2d", [sz, F64P, F64P, i32, i32, C.POINTER(KrylovParams), F64P, F64P,
                                                 C.POINTER(KrylovResult)], i32)
            self._smooth = fn("mg_smooth", [sz, dbl, F64P, F64P, i32])
            self._resid = fn("mg_residual", [sz, dbl, F64P, F64P, F64P])
            self._restrict = fn("mg_restrict", [sz, F64P, F64P])
            self._prolong = fn("mg_prolong_add", [sz, F64P, F64P])
            self._threads = fn("max_threads", [], i32)
            self._set_threads = fn("set_threads", [i32])

    @classmethod
    def reference(cls):
        p = HERE / "_ref" / "libnuma_ref.so"
        return cls(p, "ref_") if p.exists() else None

    # ---- operator
    def eval(self, n, lam, u):
        u = _f64(u)
        out = np.empty(n ** 3)
        self._eval(n, lam, _ptr(u), _ptr(out))
        return out

    def jvp(self, n, lam, u, v, mode=0):
        u, v = _f64(u), _f64(v)
        out = np.empty(n ** 3)
        self._jvp(n, lam, _ptr(u), _ptr(v), _ptr(out), mode)
        return out

    def d2(self, n, lam, u, v, mode=0):
        u, v = _f64(u), _f64(v)
        out = np.empty(n ** 3)
        self._d2(n, lam, _ptr(u), _ptr(v), _ptr(out), mode)
        return out

    def jacobi_diag(self, n, lam, u):
        u = _f64(u)
        out = np.empty(n ** 3)
        self._jdiag(n, lam, _ptr(u), _ptr(out))
        return out

    # ---- multigrid
    def mg_levels(self, n, pre=2, post=2):
        return self._levels(n, pre, post)

    def mg_apply(self, n, r, pre=2, post=2):
        r = _f64(r)
        z = np.empty(n ** 3)
        rc = self._mg_apply(n, pre, post, _ptr(r), _ptr(z))
        if rc != 0:
            raise ValueError("PoissonMG rejected the arguments")
        return z

    def mg_smooth(self, n, h2inv, x, b, order):
        x, b = _f64(x).copy(), _f64(b)
        self._smooth(n, h2inv, _ptr(x), _ptr(b), order)
        return x

    def mg_residual(self, n, h2inv, x, b):
        x, b = _f64(x), _f64(b)
        r = np.empty(n ** 3)
        self._resid(n, h2inv, _ptr(x), _ptr(b), _ptr(r))
        return r

    def mg_restrict(self, nf, rf):
        rf = _f64(rf)
        nc = (nf - 1) // 2
        bc = np.empty(nc ** 3)
        self._restrict(nf, _ptr(rf), _ptr(bc))
        return bc

    def mg_prolong_add(self, nc, xc, xf):
        xc, xf = _f64(xc), _f64(xf).copy()
        self._prolong(nc, _ptr(xc), _ptr(xf))
        return xf

    # ---- Krylov
    def gmres_bratu3d(self, n, lam, xpt, b, rtol, restart, max_iters, precond="none", jvp_mode=0,
                      x0=None, zero_guess=True):
        xpt, b = _f64(xpt), _f64(b)
        x = np.zeros(n ** 3) if x0 is None else _f64(x0).copy()
        res = GmresResult()
        self._gmres(n, lam, _ptr(xpt), jvp_mode, PRECONDS[precond], _ptr(b), _ptr(x), rtol, restart,
                    max_iters, int(zero_guess), C.byref(res))
        return x, struct_dict(res)

    def gmres_recycle_pair(self, n, lam, xpt, b1, b2, rtol, restart, max_iters, precond="mg"):
        xpt, b1, b2 = _f64(xpt), _f64(b1), _f64(b2)
        z, u = np.empty(n ** 3), np.empty(n ** 3)
        k = C.c_size_t()
        r1, r2 = GmresResult(), GmresResult()
        self._pair(n, lam, _ptr(xpt), PRECONDS[precond], _ptr(b1), _ptr(b2), rtol, restart, max_iters,
                   _ptr(z), _ptr(u), C.byref(k), C.byref(r1), C.byref(r2))
        return z, u, k.value, struct_dict(r1), struct_dict(r2)

    def gmres_poisson_mg(self, n, b, rtol, restart, max_iters):
        b = _f64(b)
        x = np.empty(n ** 3)
        res = GmresResult()
        self._gpois(n, _ptr(b), _ptr(x), rtol, restart, max_iters, C.byref(res))
        return x, struct_dict(res)

    # ---- nonlinear drivers
    def solve(self, n, lam, method="nk", precond="mg", params: KrylovParams | None = None, x0=None):
        p = params if params is not None else default_params()
        x0 = np.zeros(n ** 3) if x0 is None else _f64(x0)
        x = np.empty(n ** 3)
        res = KrylovResult()
        rc = self._solve(n, lam, METHODS[method], PRECONDS[precond], C.byref(p), _ptr(x0), _ptr(x),
                         C.byref(res))
        if rc != 0:
            raise ValueError(f"oracle solve failed with status {rc}")
        return x, struct_dict(res)

    # ---- Burgers2D / HelmholtzMG2D
    def burgers_exact(self, n, nu, dt, amp):
        out = np.empty(2 * n * n)
        if self._bexact(n, nu, dt, amp, _ptr(out)) != 0:
            raise ValueError("Burgers2D rejected the arguments")
        return out

    def burgers_eval(self, n, nu, dt, amp, w):
        w = _f64(w)
        out = np.empty(2 * n * n)
        self._beval(n, nu, dt, amp, _ptr(w), _ptr(out))
        return out

    def burgers_jvp(self, n, nu, dt, amp, w, d, mode=0):
        w, d = _f64(w), _f64(d)
        out = np.empty(2 * n * n)
        self._bjvp(n, nu, dt, amp, _ptr(w), _ptr(d), _ptr(out), mode)
        return out

    def burgers_d2(self, n, nu, dt, amp, w, d, mode=0):
        w, d = _f64(w), _f64(d)
        out = np.empty(2 * n * n)
        self._bd2(n, nu, dt, amp, _ptr(w), _ptr(d), _ptr(out), mode)
        return out

    def hmg2d_levels(self, n, alpha, nu):
        return self._hlev(n, alpha, nu)

    def hmg2d_apply(self, n, alpha, nu, r, pre=2, post=2):
        r = _f64(r)
        z = np.empty(n * n)
        self._happly(n, alpha, nu, pre, post, _ptr(r), _ptr(z))
        return z

    def solve_burgers(self, n, nu, dt, amp, method="nk", precond="mg", params=None, x0=None):
        p = params if params is not None else default_params()
        x0 = np.zeros(2 * n * n) if x0 is None else _f64(x0)
        x = np.empty(2 * n * n)
        res = KrylovResult()
        rc = self._bsolve(n, nu, dt, amp, METHODS[method], 1 if precond == "mg" else 0, C.byref(p), _ptr(x0),
                          _ptr(x), C.byref(res))
        if rc != 0:
            raise ValueError(f"Burgers2D solve failed with status {rc}")
        return x, struct_dict(res)

    # ---- Brusselator1DStep (problems/brusselator1d.hpp) and BrusselatorJacobi
    def bruss1d_previous(self, n, dt):
        out = np.empty(2 * n)
        if self._r1prev(n, dt, _ptr(out)) != 0:
            raise ValueError("Brusselator1DStep: invalid n or dt")
        return out

    def bruss1d_eval(self, n, dt, w):
        w = _f64(w)
        out = np.empty(2 * n)
        self._r1eval(n, dt, _ptr(w), _ptr(out))
        return out

    def bruss1d_jvp(self, n, dt, w, d, mode=0):
        w, d = _f64(w), _f64(d)
        out = np.empty(2 * n)
        self._r1jvp(n, dt, _ptr(w), _ptr(d), _ptr(out), mode)
        return out

    def bruss1d_d2(self, n, dt, w, d, mode=0):
        w, d = _f64(w), _f64(d)
        out = np.empty(2 * n)
        self._r1d2(n, dt, _ptr(w), _ptr(d), _ptr(out), mode)
        return out

    def bruss1d_jacobi_apply(self, n, dt, w, r):
        w, r = _f64(w), _f64(r)
        z = np.empty(2 * n)
        self._r1jac(n, dt, _ptr(w), _ptr(r), _ptr(z))
        return z

    def solve_bruss1d(self, n, dt, method="nk", precond="jacobi", params=None, x0=None):
        """x0 None: the previous state (run_campaign's natural start)."""
        p = params if params is not None else default_params()
        x = np.empty(2 * n)
        res = KrylovResult()
        kind = 5 if precond == "jacobi" else 0
        x0p = None if x0 is None else _ptr(_f64(x0))
        rc = self._r1solve(n, dt, METHODS[method], kind, C.byref(p), x0p, _ptr(x), C.byref(res))
        if rc != 0:
            raise ValueError(f"Brusselator1D solve failed with status {rc}")
        return x, struct_dict(res)

    # ---- Brusselator2D (periodic) and its coupled-block multigrid (this project's; no reference)
    @staticmethod
    def _prm(prm):
        return _f64([prm["A"], prm["B"], prm["Du"], prm["Dv"], prm["dt"]])

    def bruss2d_eval(self, n, prm, prev, w):
        pr, prev, w = self._prm(prm), _f64(prev), _f64(w)
        out = np.empty(2 * n * n)
        self._r2eval(n, _ptr(pr), _ptr(prev), _ptr(w), _ptr(out))
        return out

    def bruss2d_jvp(self, n, prm, prev, w, d, mode=0):
        pr, prev, w, d = self._prm(prm), _f64(prev), _f64(w), _f64(d)
        out = np.empty(2 * n * n)
        self._r2jvp(n, _ptr(pr), _ptr(prev), _ptr(w), _ptr(d), _ptr(out), mode)
        return out

    def bruss2d_d2(self, n, prm, prev, w, d, mode=0):
        pr, prev, w, d = self._prm(prm), _f64(prev), _f64(w), _f64(d)
        out = np.empty(2 * n * n)
        self._r2d2(n, _ptr(pr), _ptr(prev), _ptr(w), _ptr(d), _ptr(out), mode)
        return out

    def bmg2d_levels(self, n):
        return self._bmglev(n)

    def bmg2d_apply(self, n, prm, w, r, pre=2, post=2):
        pr, w, r = self._prm(prm), _f64(w), _f64(r)
        z = np.empty(2 * n * n)
        if self._bmgapply(n, _ptr(pr), _ptr(w), pre, post, _ptr(r), _ptr(z)) != 0:
            raise ValueError("BrussMG2D needs an even n >= 4")
        return z

    def solve_bruss2d(self, n, prm, prev, method="nk", precond="mg", params=None, x0=None):
        p = params if params is not None else default_params()
        pr, prev = self._prm(prm), _f64(prev)
        x = np.empty(2 * n * n)
        res = KrylovResult()
        kind = 6 if precond == "mg" else 0
        x0p = None if x0 is None else _ptr(_f64(x0))
        rc = self._r2solve(n, _ptr(pr), _ptr(prev), METHODS[method], kind, C.byref(p), x0p, _ptr(x), C.byref(res))
        if rc != 0:
            raise ValueError(f"Brusselator2D solve failed with status {rc}")
        return x, struct_dict(res)

    def forcing(self, params, k, rnorm, rprev, eta_prev, res0):
        return self._forcing(C.byref(params), k, rnorm, rprev, eta_prev, res0)

    def max_threads(self):
        return self._threads()

    def set_threads(self, t):
        self._set_threads(t)
