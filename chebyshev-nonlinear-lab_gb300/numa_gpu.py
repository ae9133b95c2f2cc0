"""Python binding of libnuma_gpu.so (ctypes over the C ABI of include/numa_gpu.h).

The objects mirror the reference's C++ interfaces (namespace numa::op):
``Bratu3D`` (eval / jvp / d2 / jacobi_diag), ``Burgers2D`` (eval / jvp / d2 / exact),
``PoissonMG`` and ``HelmholtzMG2D`` (V-cycles), preconditioner ``Provider`` objects
(make / apply), ``gmres`` / ``gmres_recycled`` and the drivers ``newton_krylov``,
``chebyshev_inexact`` and ``tf_chebyshev_2018`` on either operator.  Vectors live on the GPU
(``Vec``); ``Vec.from_numpy`` / ``Vec.numpy`` move them to and from host memory.

There is no CPU fallback: loading fails loudly when the library has not been built, and every
call that needs a GPU raises ``NumaGPUError`` when there is none.
"""
from __future__ import annotations

import atexit
import ctypes as C
import os
import weakref
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("NUMA_GPU_LIB", HERE / "libnuma_gpu.so"))

# enums (include/numa_gpu.h)
OK = 0
FP64, FP32 = 0, 1
ANALYTIC, FD, ANALYTIC_FP32, ANALYTIC_FP32X = 0, 1, 2, 3
MGS, CGS2, CGS1 = 0, 1, 2
METHODS = {"nk": 0, "cheb": 1, "rec": 2, "tf2018": 3}
PRECONDS = {"none": 0, "mg": 1, "jacobi": 2, "burgers_mg": 3, "bruss_jacobi": 5, "bruss_mg": 6, "jacobian_mg": 7}


class KrylovParams(C.Structure):
    """numa_krylov_params: KrylovParams (methods/krylov_newton.hpp:24-38) plus extensions."""
    _fields_ = [
        ("rtol_nl", C.c_double), ("max_nl", C.c_uint64), ("eta_init", C.c_double),
        ("eta_max", C.c_double), ("gamma", C.c_double), ("alpha", C.c_double),
        ("eta2_factor", C.c_double), ("eta2_max", C.c_double), ("gmres_restart", C.c_uint64),
        ("gmres_max_iters", C.c_uint64), ("armijo", C.c_double), ("min_lambda", C.c_double),
        ("recycle", C.c_int32), ("jvp_mode", C.c_int32), ("d2_mode", C.c_int32),
        ("orth", C.c_int32), ("flexible", C.c_int32), ("jvp_precision", C.c_int32),
        ("jvp_tight", C.c_int32), ("coarse_jacobian", C.c_int32), ("reserved", C.c_int32 * 2),
    ]


class LearnedTrainParams(C.Structure):
    """numa_learned_train_params"""
    _fields_ = [
        ("n_fine", C.c_size_t), ("lambda_min", C.c_double), ("lambda_max", C.c_double),
        ("instances", C.c_int32), ("states", C.c_int32), ("rhs_per_state", C.c_int32), ("krylov_per_state", C.c_int32),
        ("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float), ("seed", C.c_uint64),
        ("solve_rtol", C.c_double),
    ]


class LearnedTrainReport(C.Structure):
    """numa_learned_train_report"""
    _fields_ = [("samples", C.c_size_t), ("gen_seconds", C.c_double), ("train_seconds", C.c_double),
                ("loss_first", C.c_float), ("loss_last", C.c_float), ("target_ms", C.c_float)]


class BrusselatorParams(C.Structure):
    """numa_brusselator2d_params of include/numa_gpu.h."""
    _fields_ = [("A", C.c_double), ("B", C.c_double), ("Du", C.c_double), ("Dv", C.c_double), ("dt", C.c_double)]


def brusselator_params(A: float = 1.0, B: float = 3.4, Du: float = 0.002, Dv: float = 0.002,
                       dt: float = 0.01) -> BrusselatorParams:
    """The 2-species 2048^2 configuration's parameters by default."""
    return BrusselatorParams(A, B, Du, Dv, dt)


class BatchInstance(C.Structure):
    _fields_ = [("n", C.c_size_t), ("lambda_", C.c_double)]


class BatchResult(C.Structure):
    _fields_ = [("converged", C.c_int32), ("status", C.c_int32), ("iters", C.c_uint64), ("n_F", C.c_uint64),
                ("n_JVP", C.c_uint64), ("n_lin_iters", C.c_uint64), ("n_prec", C.c_uint64), ("res_rel", C.c_double),
                ("seconds", C.c_double)]


class BatchTuning(C.Structure):
    """numa_batch_tuning: tile shapes of the batched solver."""
    _fields_ = [("planes", C.c_int32), ("elems_per_block", C.c_int32), ("reserved", C.c_int32 * 6)]


class KrylovResult(C.Structure):
    """numa_krylov_result: KrylovResult (krylov_newton.hpp:40-49) plus timers."""
    _fields_ = [
        ("converged", C.c_int32), ("status", C.c_int32), ("iters", C.c_uint64),
        ("n_F", C.c_uint64), ("n_JVP", C.c_uint64), ("n_D2", C.c_uint64),
        ("n_lin_iters", C.c_uint64), ("n_lin_failures", C.c_uint64), ("n_prec", C.c_uint64),
        ("res0", C.c_double), ("res", C.c_double), ("t_F", C.c_double), ("t_JVP", C.c_double),
        ("t_D2", C.c_double), ("t_prec", C.c_double), ("t_setup_dynamic", C.c_double),
        ("t_total", C.c_double),
    ]


class GmresResult(C.Structure):
    """numa_gmres_result: GmresResult (linalg/gmres.hpp:14-21)."""
    _fields_ = [
        ("iters", C.c_uint64), ("matvecs", C.c_uint64), ("precs", C.c_uint64),
        ("rel_res", C.c_double), ("converged", C.c_int32), ("breakdown", C.c_int32),
    ]


def to_dict(s) -> dict:
    return {name: getattr(s, name) for name, _ in s._fields_ if name != "reserved"}


APPLY_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p)
PRECOND_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p)

_P = C.c_void_p
_PP = C.POINTER(C.c_void_p)
_SZ = C.c_size_t
_D = C.c_double
_I = C.c_int
_F64P = C.POINTER(C.c_double)
_F32P = C.POINTER(C.c_float)

# name -> (argtypes, restype)
SIGNATURES = {
    "numa_gpu_abi_version": ([], _I),
    "numa_gpu_status_string": ([_I], C.c_char_p),
    "numa_krylov_params_default": ([C.POINTER(KrylovParams)], None),
    "numa_gpu_ctx_create": ([_I, _PP], _I),
    "numa_gpu_ctx_destroy": ([_P], _I),
    "numa_gpu_ctx_synchronize": ([_P], _I),
    "numa_gpu_ctx_last_error": ([_P], C.c_char_p),
    "numa_gpu_ctx_set_timing": ([_P, _I], _I),
    "numa_gpu_ctx_kernel_launches": ([_P, C.POINTER(C.c_uint64)], _I),
    "numa_gpu_ctx_reset_kernel_launches": ([_P], _I),
    "numa_gpu_ctx_stream": ([_P, _PP], _I),
    "numa_gpu_vec_create": ([_P, _SZ, _PP], _I),
    "numa_gpu_vec_destroy": ([_P], _I),
    "numa_gpu_vec_size": ([_P, C.POINTER(_SZ)], _I),
    "numa_gpu_vec_device_ptr": ([_P, _PP], _I),
    "numa_gpu_vec_upload": ([_P, _F64P, _SZ], _I),
    "numa_gpu_vec_download": ([_P, _F64P, _SZ], _I),
    "numa_gpu_vec_fill": ([_P, _D], _I),
    "numa_gpu_vec_copy": ([_P, _P], _I),
    "numa_gpu_vec_dot": ([_P, _P, _F64P], _I),
    "numa_gpu_vec_norm2": ([_P, _F64P], _I),
    "numa_gpu_vec_axpy": ([_D, _P, _P], _I),
    "numa_gpu_bratu3d_create": ([_P, _SZ, _D, _PP], _I),
    "numa_gpu_bratu3d_destroy": ([_P], _I),
    "numa_gpu_bratu3d_size": ([_P, C.POINTER(_SZ)], _I),
    "numa_gpu_bratu3d_eval": ([_P, _P, _P], _I),
    "numa_gpu_bratu3d_jvp": ([_P, _P, _P, _P, _I], _I),
    "numa_gpu_bratu3d_d2": ([_P, _P, _P, _P, _I], _I),
    "numa_gpu_bratu3d_jacobi_diag": ([_P, _P, _P], _I),
    "numa_gpu_burgers2d_create": ([_P, _SZ, _D, _D, _D, _PP], _I),
    "numa_gpu_burgers2d_destroy": ([_P], _I),
    "numa_gpu_burgers2d_size": ([_P, C.POINTER(_SZ)], _I),
    "numa_gpu_burgers2d_cell_reynolds": ([_P, _F64P], _I),
    "numa_gpu_burgers2d_exact": ([_P, _P], _I),
    "numa_gpu_burgers2d_eval": ([_P, _P, _P], _I),
    "numa_gpu_burgers2d_jvp": ([_P, _P, _P, _P, _I], _I),
    "numa_gpu_burgers2d_d2": ([_P, _P, _P, _P, _I], _I),
    "numa_gpu_burgers2d_solve": ([_P, _I, _P, C.POINTER(KrylovParams), _P, C.POINTER(KrylovResult)], _I),
    "numa_gpu_hmg2d_create": ([_P, _SZ, _D, _D, _I, _I, _PP], _I),
    "numa_gpu_hmg2d_destroy": ([_P], _I),
    "numa_gpu_hmg2d_levels": ([_P, C.POINTER(_SZ)], _I),
    "numa_gpu_hmg2d_apply": ([_P, _P, _P], _I),
    "numa_gpu_brusselator1d_create": ([_P, _SZ, _D, _PP], _I),
    "numa_gpu_brusselator1d_destroy": ([_P], _I),
    "numa_gpu_brusselator1d_size": ([_P, C.POINTER(_SZ)], _I),
    "numa_gpu_brusselator1d_previous": ([_P, _P], _I),
    "numa_gpu_brusselator1d_eval": ([_P, _P, _P], _I),
    "numa_gpu_brusselator1d_jvp": ([_P, _P, _P, _P, _I], _I),
    "numa_gpu_brusselator1d_d2": ([_P, _P, _P, _P, _I], _I),
    "numa_gpu_brusselator1d_solve": ([_P, _I, _P, C.POINTER(KrylovParams), _P, C.POINTER(KrylovResult)], _I),
    "numa_gpu_provider_create_brusselator_jacobi": ([_P, _PP], _I),
    "numa_gpu_solve_brusselator1d_host": ([_P, _SZ, _D, _I, _I, C.POINTER(KrylovParams), _F64P, _F64P,
                                           C.POINTER(KrylovResult)], _I),
    "numa_gpu_brusselator2d_create": ([_P, _SZ, C.POINTER(BrusselatorParams), _PP], _I),
    "numa_gpu_brusselator2d_destroy": ([_P], _I),
    "numa_gpu_brusselator2d_size": ([_P, C.POINTER(_SZ)], _I),
    "numa_gpu_brusselator2d_set_previous": ([_P, _P], _I),
    "numa_gpu_brusselator2d_eval": ([_P, _P, _P], _I),
    "numa_gpu_brusselator2d_jvp": ([_P, _P, _P, _P, _I], _I),
    "numa_gpu_brusselator2d_d2": ([_P, _P, _P, _P, _I], _I),
    "numa_gpu_brusselator2d_solve": ([_P, _I, _P, C.POINTER(KrylovParams), _P, C.POINTER(KrylovResult)], _I),
    "numa_gpu_brusselator2d_advance": ([_P, _I, _SZ, _P, C.POINTER(KrylovParams), _P, C.POINTER(KrylovResult)], _I),
    "numa_gpu_provider_create_brusselator_mg": ([_P, _I, _I, _I, _PP], _I),
    "numa_gpu_brusselator2d_advance_host": ([_P, _SZ, C.POINTER(BrusselatorParams), _SZ, _I, _I, _I,
                                             C.POINTER(KrylovParams), _F64P, _F64P, C.POINTER(KrylovResult)], _I),
    "numa_gpu_bmg2d_create": ([_P, _SZ, C.POINTER(BrusselatorParams), _I, _I, _I, _PP], _I),
    "numa_gpu_bmg2d_destroy": ([_P], _I),
    "numa_gpu_bmg2d_levels": ([_P, C.POINTER(_SZ)], _I),
    "numa_gpu_bmg2d_set_state": ([_P, _P], _I),
    "numa_gpu_bmg2d_apply": ([_P, _P, _P], _I),
    "numa_gpu_provider_create_burgers_mg": ([_P, _SZ, _D, _D, _PP], _I),
    "numa_gpu_solve_burgers2d_host": ([_P, _SZ, _D, _D, _D, _I, _I, C.POINTER(KrylovParams), _F64P, _F64P,
                                       C.POINTER(KrylovResult)], _I),
    "numa_gpu_mg_create": ([_P, _SZ, _I, _I, _PP], _I),
    "numa_gpu_mg_create_ex": ([_P, _SZ, _I, _I, _I, _I, _PP], _I),
    "numa_gpu_mg_destroy": ([_P], _I),
    "numa_gpu_mg_levels": ([_P, C.POINTER(_SZ)], _I),
    "numa_gpu_mg_apply": ([_P, _P, _P], _I),
    "numa_gpu_provider_create_identity": ([_P, _PP], _I),
    "numa_gpu_provider_create_poisson_mg": ([_P, _SZ, _I, _I, _I, _PP], _I),
    "numa_gpu_provider_create_jacobi": ([_P, _PP], _I),
    "numa_gpu_provider_destroy": ([_P], _I),
    "numa_gpu_provider_make": ([_P, _P], _I),
    "numa_gpu_provider_apply": ([_P, _P, _P], _I),
    "numa_gpu_krylov_space_create": ([_P, _PP], _I),
    "numa_gpu_krylov_space_destroy": ([_P], _I),
    "numa_gpu_krylov_space_k": ([_P, C.POINTER(_SZ)], _I),
    "numa_gpu_gmres": ([_P, APPLY_FN, _P, PRECOND_FN, _P, _P, _P, _D, _SZ, _SZ, _I, _I, _I, _P, _P,
                        C.POINTER(GmresResult)], _I),
    "numa_gpu_gmres_bratu3d": ([_P, _P, _I, _P, _P, _P, _D, _SZ, _SZ, _I, _I, _I, _P, _P,
                                C.POINTER(GmresResult)], _I),
    "numa_gpu_gmres_recycled_bratu3d": ([_P, _P, _I, _P, _P, _P, _D, _SZ, _SZ, _I, _P, _P,
                                         C.POINTER(GmresResult)], _I),
    "numa_gpu_forcing": ([C.POINTER(KrylovParams), _SZ, _D, _D, _D, _D], _D),
    "numa_gpu_newton_krylov": ([_P, _P, C.POINTER(KrylovParams), _P, C.POINTER(KrylovResult)], _I),
    "numa_gpu_chebyshev_inexact": ([_P, _P, C.POINTER(KrylovParams), _P, C.POINTER(KrylovResult)], _I),
    "numa_gpu_tf_chebyshev_2018": ([_P, _P, C.POINTER(KrylovParams), _P, C.POINTER(KrylovResult)], _I),
    "numa_gpu_solve_bratu3d_host": ([_P, _SZ, _D, _I, _I, _I, C.POINTER(KrylovParams), _F64P, _F64P,
                                     C.POINTER(KrylovResult)], _I),
    "numa_gpu_mg_apply_noalloc": ([_SZ, _I, _I, _P, _P, _P], _I),
    "numa_gpu_diag_fp64_peak": ([_P, _F64P], _I),
    "numa_gpu_diag_time_smoother": ([_P, _I, _F64P], _I),
    "numa_gpu_diag_time_eval": ([_P, _P, _I, _I, _F64P], _I),
    "numa_gpu_diag_eval": ([_P, _P, _I, _P, _F64P], _I),
    "numa_gpu_diag_time_bmg2d_pass": ([_P, _I, _F64P], _I),
    "numa_gpu_diag_exp": ([_P, _P, _P], _I),
    "numa_gpu_diag_div": ([_P, C.c_double, _P], _I),
    "numa_gpu_diag_conv3d": ([_P, _SZ, _I, _I, _I, _F32P, _F32P, _F32P, _F32P], _I),
    "numa_gpu_diag_conv3d_wgrad": ([_P, _SZ, _I, _I, _F32P, _F32P, _F32P, _F32P], _I),
    "numa_gpu_solve_batch": ([_I, C.POINTER(BatchInstance), _SZ, _I, _I, C.POINTER(KrylovParams), _I,
                              C.POINTER(BatchResult), _F64P], _I),
    "numa_gpu_batch_last_error": ([], C.c_char_p),
    "numa_gpu_batch_create": ([_I, _I, _PP], _I),
    "numa_gpu_batch_destroy": ([_P], _I),
    "numa_gpu_batch_set_workers": ([_P, _I], _I),
    "numa_gpu_batch_autotune": ([_P, C.POINTER(BatchInstance), _SZ, _I, _I, C.POINTER(KrylovParams),
                                 C.POINTER(_I), _I, C.POINTER(_I), _F64P], _I),
    "numa_gpu_batch_solve": ([_P, C.POINTER(BatchInstance), _SZ, _I, _I, C.POINTER(KrylovParams),
                              C.POINTER(BatchResult), _F64P], _I),
    "numa_gpu_learned_create": ([_P, _SZ, C.c_uint64, _PP], _I),
    "numa_gpu_learned_destroy": ([_P], _I),
    "numa_gpu_learned_num_params": ([_P, C.POINTER(_SZ)], _I),
    "numa_gpu_learned_get_params": ([_P, _F32P, _SZ], _I),
    "numa_gpu_learned_set_params": ([_P, _F32P, _SZ], _I),
    "numa_gpu_learned_forward": ([_P, _F32P, _F32P], _I),
    "numa_gpu_learned_gradient": ([_P, _F32P, _F32P, _F32P, _F32P], _I),
    "numa_gpu_learned_train": ([_P, C.POINTER(LearnedTrainParams), C.POINTER(LearnedTrainReport)], _I),
    "numa_gpu_provider_create_learned": ([_P, _SZ, _P, _D, _PP], _I),
    "numa_gpu_provider_learned_stats": ([_P, C.POINTER(_SZ), C.POINTER(_SZ)], _I),
    "numa_gpu_provider_create_jacobian_mg": ([_P, _SZ, _I, _I, _PP], _I),
    "numa_gpu_bsolver_create": ([_P, C.POINTER(BatchInstance), _SZ, C.POINTER(KrylovParams), _PP], _I),
    "numa_gpu_bsolver_destroy": ([_P], _I),
    "numa_gpu_bsolver_solve": ([_P, _F64P, C.POINTER(BatchResult), _F64P], _I),
    "numa_gpu_bsolver_get_tuning": ([_P, C.POINTER(BatchTuning)], _I),
    "numa_gpu_bsolver_set_tuning": ([_P, C.POINTER(BatchTuning)], _I),
    "numa_gpu_bsolver_autotune": ([_P, C.POINTER(C.c_int), _I, C.POINTER(C.c_int), _I, C.POINTER(BatchTuning),
                                   _F64P], _I),
}

_lib = None


def load(path: str | Path | None = None) -> C.CDLL:
    """Loads libnuma_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} not found: build it with chebyshev-nonlinear-lab_gb300/build.py")
    lib = C.CDLL(str(p))
    for name, (args, res) in SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    if path is None:
        _lib = lib
    return lib


class NumaGPUError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        lib = load()
        msg = f"{where}: {lib.numa_gpu_status_string(code).decode()} ({code})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


def default_params(**kw) -> KrylovParams:
    """KrylovParams{} (methods/krylov_newton.hpp:24-38) with keyword overrides."""
    p = KrylovParams()
    load().numa_krylov_params_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


# Contexts still open when the interpreter exits are closed (their objects first) by an exit hook, which
# runs before the CUDA runtime is torn down: finalisers left to module teardown could otherwise free
# device memory after it.
_live_contexts: "weakref.WeakSet" = weakref.WeakSet()  # contexts and batch executors


def _ctx_open(ctx) -> bool:
    """Whether a child object may still call its C destroy function.  Objects close before their context
    (Context.close closes them first), except when the context and its children become garbage together:
    the collector clears the context's weak references to them before it runs any finalizer, in no fixed
    order, so a child can be finalised after the context's C handle is gone.  Its C handle then points at
    a destroyed context and is dropped without a call (its device memory is released with the process)."""
    return bool(getattr(ctx, "h", None))


@atexit.register
def _close_live_contexts():
    for ctx in list(_live_contexts):
        try:
            ctx.close()
        except Exception:
            pass


class Context:
    """One device and one stream (numa_gpu_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.numa_gpu_ctx_create(device, C.byref(h))
        if rc != OK:
            raise NumaGPUError(rc, "numa_gpu_ctx_create")
        self.h = h
        self._children = weakref.WeakSet()
        _live_contexts.add(self)

    def _adopt(self, obj):
        """Objects created on this context are closed before it (whatever the order of garbage collection)."""
        self._children.add(obj)

    def check(self, rc: int, where: str):
        if rc != OK:
            raise NumaGPUError(rc, where, self.lib.numa_gpu_ctx_last_error(self.h).decode())

    def close(self):
        if self.h:
            for child in list(self._children):
                try:
                    child.close()
                except Exception:
                    pass
            self.lib.numa_gpu_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        self.check(self.lib.numa_gpu_ctx_synchronize(self.h), "synchronize")

    def set_timing(self, on: bool):
        self.check(self.lib.numa_gpu_ctx_set_timing(self.h, int(on)), "set_timing")

    def kernel_launches(self) -> int:
        v = C.c_uint64()
        self.check(self.lib.numa_gpu_ctx_kernel_launches(self.h, C.byref(v)), "kernel_launches")
        return v.value

    def reset_kernel_launches(self):
        self.check(self.lib.numa_gpu_ctx_reset_kernel_launches(self.h), "reset_kernel_launches")

    def stream(self) -> int:
        s = C.c_void_p()
        self.check(self.lib.numa_gpu_ctx_stream(self.h, C.byref(s)), "stream")
        return s.value or 0

    def fp64_peak_tflops(self) -> float:
        """Measured FP64 FMA throughput of this GPU (diagnostic)."""
        v = C.c_double()
        self.check(self.lib.numa_gpu_diag_fp64_peak(self.h, C.byref(v)), "diag_fp64_peak")
        return v.value

    def vec(self, n: int) -> "Vec":
        return Vec(self, n)

    def from_numpy(self, a) -> "Vec":
        a = _f64(a).ravel()
        v = Vec(self, a.size)
        v.upload(a)
        return v


class Vec:
    """A device FP64 vector (numa_gpu_vec); the reference's DVec on the GPU."""

    def __init__(self, ctx: Context, n: int, handle=None):
        self.ctx = ctx
        self.lib = ctx.lib
        self.n = int(n)
        if handle is None:
            h = C.c_void_p()
            ctx.check(self.lib.numa_gpu_vec_create(ctx.h, self.n, C.byref(h)), "vec_create")
            self.h = h
            self.owned = True
            ctx._adopt(self)
        else:
            self.h = C.c_void_p(handle)
            self.owned = False

    def close(self):
        if self.owned and self.h:
            if _ctx_open(self.ctx):
                self.lib.numa_gpu_vec_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, a):
        a = _f64(a).ravel()
        self.ctx.check(self.lib.numa_gpu_vec_upload(self.h, a.ctypes.data_as(_F64P), a.size), "vec_upload")
        return self

    def numpy(self) -> np.ndarray:
        out = np.empty(self.n)
        self.ctx.check(self.lib.numa_gpu_vec_download(self.h, out.ctypes.data_as(_F64P), self.n), "vec_download")
        return out

    def fill(self, v: float):
        self.ctx.check(self.lib.numa_gpu_vec_fill(self.h, float(v)), "vec_fill")
        return self

    def copy_from(self, src: "Vec"):
        self.ctx.check(self.lib.numa_gpu_vec_copy(src.h, self.h), "vec_copy")
        return self

    def dot(self, other: "Vec") -> float:
        out = C.c_double()
        self.ctx.check(self.lib.numa_gpu_vec_dot(self.h, other.h, C.byref(out)), "vec_dot")
        return out.value

    def norm2(self) -> float:
        out = C.c_double()
        self.ctx.check(self.lib.numa_gpu_vec_norm2(self.h, C.byref(out)), "vec_norm2")
        return out.value

    def axpy(self, a: float, x: "Vec"):
        """self += a * x"""
        self.ctx.check(self.lib.numa_gpu_vec_axpy(float(a), x.h, self.h), "vec_axpy")
        return self

    def device_ptr(self) -> int:
        p = C.c_void_p()
        self.ctx.check(self.lib.numa_gpu_vec_device_ptr(self.h, C.byref(p)), "vec_device_ptr")
        return p.value or 0


class Bratu3D:
    """Bratu3D(n, lambda) (problems/bratu3d.hpp:12-16) on the GPU."""

    def __init__(self, ctx: Context, n: int, lam: float = 1.0):
        self.ctx, self.lib, self.n, self.lam = ctx, ctx.lib, int(n), float(lam)
        h = C.c_void_p()
        ctx.check(self.lib.numa_gpu_bratu3d_create(ctx.h, self.n, self.lam, C.byref(h)), "bratu3d_create")
        self.h = h
        self.ctx._adopt(self)

    def close(self):
        if self.h and _ctx_open(self.ctx):
            self.lib.numa_gpu_bratu3d_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def size(self) -> int:
        return self.n ** 3

    def eval(self, x: Vec, out: Vec):
        self.ctx.check(self.lib.numa_gpu_bratu3d_eval(self.h, x.h, out.h), "bratu3d_eval")

    def jvp(self, x: Vec, v: Vec, out: Vec, mode: int = ANALYTIC):
        self.ctx.check(self.lib.numa_gpu_bratu3d_jvp(self.h, x.h, v.h, out.h, mode), "bratu3d_jvp")

    def d2(self, x: Vec, v: Vec, out: Vec, mode: int = ANALYTIC):
        self.ctx.check(self.lib.numa_gpu_bratu3d_d2(self.h, x.h, v.h, out.h, mode), "bratu3d_d2")

    def jacobi_diag(self, x: Vec, d: Vec):
        self.ctx.check(self.lib.numa_gpu_bratu3d_jacobi_diag(self.h, x.h, d.h), "bratu3d_jacobi_diag")

    def eval_as(self, x: Vec, out: Vec, precision: int = FP64) -> float:
        """out = F(x) as the drivers' evaluation at that precision forms it (FP32: the mixed path's);
        returns ||F(x)|| (diagnostic)."""
        v = C.c_double()
        self.ctx.check(self.lib.numa_gpu_diag_eval(self.h, x.h, precision, out.h, C.byref(v)), "diag_eval")
        return v.value

    def time_eval(self, x: Vec, precision: int = FP64, reps: int = 20) -> float:
        """Average ms of one residual evaluation with its fused norm and cache (diagnostic)."""
        v = C.c_double()
        self.ctx.check(self.lib.numa_gpu_diag_time_eval(self.h, x.h, precision, reps, C.byref(v)), "diag_time_eval")
        return v.value


class Burgers2D:
    """Burgers2D(n, nu, dt, amplitude) (problems/burgers2d.hpp:23-52) on the GPU; N = 2 n^2."""

    def __init__(self, ctx: Context, n: int, nu: float, dt: float, amplitude: float = 1.0):
        self.ctx, self.lib, self.n = ctx, ctx.lib, int(n)
        self.nu, self.dt, self.amplitude = float(nu), float(dt), float(amplitude)
        h = C.c_void_p()
        ctx.check(self.lib.numa_gpu_burgers2d_create(ctx.h, self.n, self.nu, self.dt, self.amplitude, C.byref(h)),
                  "burgers2d_create")
        self.h = h
        self.ctx._adopt(self)

    def close(self):
        if self.h and _ctx_open(self.ctx):
            self.lib.numa_gpu_burgers2d_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def size(self) -> int:
        return 2 * self.n * self.n

    def cell_reynolds(self) -> float:
        v = C.c_double()
        self.ctx.check(self.lib.numa_gpu_burgers2d_cell_reynolds(self.h, C.byref(v)), "burgers2d_cell_reynolds")
        return v.value

    def exact(self, out: Vec):
        self.ctx.check(self.lib.numa_gpu_burgers2d_exact(self.h, out.h), "burgers2d_exact")

    def eval(self, w: Vec, out: Vec):
        self.ctx.check(self.lib.numa_gpu_burgers2d_eval(self.h, w.h, out.h), "burgers2d_eval")

    def jvp(self, w: Vec, d: Vec, out: Vec, mode: int = ANALYTIC):
        self.ctx.check(self.lib.numa_gpu_burgers2d_jvp(self.h, w.h, d.h, out.h, mode), "burgers2d_jvp")

    def d2(self, w: Vec, d: Vec, out: Vec, mode: int = ANALYTIC):
        self.ctx.check(self.lib.numa_gpu_burgers2d_d2(self.h, w.h, d.h, out.h, mode), "burgers2d_d2")


class _Handle:
    """A C handle with a destroy function, closed before its context."""
    _destroy = ""

    def close(self):
        if getattr(self, "h", None) and _ctx_open(getattr(self, "ctx", None)):
            getattr(self.lib, self._destroy)(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Brusselator1D(_Handle):
    """Brusselator1DStep(n, dt) (problems/brusselator1d.hpp:22-45) on the GPU; N = 2 n."""
    _destroy = "numa_gpu_brusselator1d_destroy"

    def __init__(self, ctx: Context, n: int, dt: float):
        self.ctx, self.lib, self.n, self.dt = ctx, ctx.lib, int(n), float(dt)
        h = C.c_void_p()
        ctx.check(self.lib.numa_gpu_brusselator1d_create(ctx.h, self.n, self.dt, C.byref(h)), "brusselator1d_create")
        self.h = h
        self.ctx._adopt(self)

    def size(self) -> int:
        return 2 * self.n

    def previous(self, out: Vec):
        self.ctx.check(self.lib.numa_gpu_brusselator1d_previous(self.h, out.h), "brusselator1d_previous")

    def eval(self, w: Vec, out: Vec):
        self.ctx.check(self.lib.numa_gpu_brusselator1d_eval(self.h, w.h, out.h), "brusselator1d_eval")

    def jvp(self, w: Vec, d: Vec, out: Vec, mode: int = ANALYTIC):
        self.ctx.check(self.lib.numa_gpu_brusselator1d_jvp(self.h, w.h, d.h, out.h, mode), "brusselator1d_jvp")

    def d2(self, w: Vec, d: Vec, out: Vec, mode: int = ANALYTIC):
        self.ctx.check(self.lib.numa_gpu_brusselator1d_d2(self.h, w.h, d.h, out.h, mode), "brusselator1d_d2")


class Brusselator2D(_Handle):
    """Implicit-Euler step of the periodic 2-species Brusselator on n x n; N = 2 n^2."""
    _destroy = "numa_gpu_brusselator2d_destroy"

    def __init__(self, ctx: Context, n: int, params: BrusselatorParams | None = None):
        self.ctx, self.lib, self.n = ctx, ctx.lib, int(n)
        self.params = params if params is not None else brusselator_params()
        h = C.c_void_p()
        ctx.check(self.lib.numa_gpu_brusselator2d_create(ctx.h, self.n, C.byref(self.params), C.byref(h)),
                  "brusselator2d_create")
        self.h = h
        self.ctx._adopt(self)

    def size(self) -> int:
        return 2 * self.n * self.n

    def set_previous(self, w: Vec):
        self.ctx.check(self.lib.numa_gpu_brusselator2d_set_previous(self.h, w.h), "brusselator2d_set_previous")

    def eval(self, w: Vec, out: Vec):
        self.ctx.check(self.lib.numa_gpu_brusselator2d_eval(self.h, w.h, out.h), "brusselator2d_eval")

    def jvp(self, w: Vec, d: Vec, out: Vec, mode: int = ANALYTIC):
        self.ctx.check(self.lib.numa_gpu_brusselator2d_jvp(self.h, w.h, d.h, out.h, mode), "brusselator2d_jvp")

    def d2(self, w: Vec, d: Vec, out: Vec, mode: int = ANALYTIC):
        self.ctx.check(self.lib.numa_gpu_brusselator2d_d2(self.h, w.h, d.h, out.h, mode), "brusselator2d_d2")

    def advance(self, x: Vec, steps: int, method: str = "nk", params: KrylovParams | None = None,
                provider: "Provider | None" = None) -> list[dict]:
        """`steps` implicit-Euler steps from the state x (overwritten); one result per step."""
        p = params if params is not None else default_params()
        if method == "rec":
            p.recycle = 1
        res = (KrylovResult * steps)()
        rc = self.lib.numa_gpu_brusselator2d_advance(self.h, METHODS[method], steps, x.h, C.byref(p),
                                                     provider.h if provider else None, res)
        self.ctx.check(rc, "brusselator2d_advance")
        return [to_dict(r) for r in res]


class BrussMG2D(_Handle):
    """The coupled-block periodic multigrid of Brusselator2D: set_state(w), then apply(r, z)."""
    _destroy = "numa_gpu_bmg2d_destroy"

    def __init__(self, ctx: Context, n: int, params: BrusselatorParams | None = None, precision: int = FP64,
                 pre: int = 2, post: int = 2):
        self.ctx, self.lib, self.n = ctx, ctx.lib, int(n)
        self.params = params if params is not None else brusselator_params()
        h = C.c_void_p()
        ctx.check(self.lib.numa_gpu_bmg2d_create(ctx.h, self.n, C.byref(self.params), precision, pre, post,
                                                 C.byref(h)), "bmg2d_create")
        self.h = h
        self.ctx._adopt(self)

    def levels(self) -> int:
        v = C.c_size_t()
        self.ctx.check(self.lib.numa_gpu_bmg2d_levels(self.h, C.byref(v)), "bmg2d_levels")
        return v.value

    def set_state(self, w: Vec):
        self.ctx.check(self.lib.numa_gpu_bmg2d_set_state(self.h, w.h), "bmg2d_set_state")

    def apply(self, r: Vec, z: Vec):
        self.ctx.check(self.lib.numa_gpu_bmg2d_apply(self.h, r.h, z.h), "bmg2d_apply")

    def time_pass(self, reps: int = 20) -> float:
        """ms of one finest-level colour pass (after set_state)."""
        v = C.c_double()
        self.ctx.check(self.lib.numa_gpu_diag_time_bmg2d_pass(self.h, reps, C.byref(v)), "diag_time_bmg2d_pass")
        return v.value


def batch_config_instances(count: int = 128, seed: int = 42, sizes=(31, 63, 127),
                           lam_range=(1.0, 6.5)) -> list[tuple[int, float]]:
    """The batched configuration's instance table: `count` Bratu3D instances (n, lambda), n drawn
    uniformly from `sizes` and lambda ~ U[lam_range] from numpy's PCG64 stream of `seed` (all n
    first, then all lambda)."""
    rng = np.random.default_rng(seed)
    ns = rng.choice(list(sizes), count)
    lams = rng.uniform(lam_range[0], lam_range[1], count)
    return [(int(n), float(lm)) for n, lm in zip(ns, lams)]


def brusselator2d_initial(n: int, A: float = 1.0, B: float = 3.4, seed: int = 20261203) -> np.ndarray:
    """u = A + 0.01 N(0,1), v = B/A + 0.01 N(0,1) per point from numpy's PCG64 stream of `seed`
    (2 n^2 normals: the u plane first)."""
    z = np.random.default_rng(seed).standard_normal(2 * n * n)
    z[: n * n] = A + 0.01 * z[: n * n]
    z[n * n:] = B / A + 0.01 * z[n * n:]
    return z


class HelmholtzMG2D:
    """HelmholtzMG2D(n, alpha, nu, pre, post) (linalg/helmholtz_mg2d.hpp:13-32): one V-cycle per call."""

    def __init__(self, ctx: Context, n: int, alpha: float, nu: float, pre: int = 2, post: int = 2):
        self.ctx, self.lib, self.n = ctx, ctx.lib, int(n)
        h = C.c_void_p()
        ctx.check(self.lib.numa_gpu_hmg2d_create(ctx.h, self.n, float(alpha), float(nu), pre, post, C.byref(h)),
                  "hmg2d_create")
        self.h = h
        self.ctx._adopt(self)

    def close(self):
        if self.h and _ctx_open(self.ctx):
            self.lib.numa_gpu_hmg2d_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def levels(self) -> int:
        v = C.c_size_t()
        self.ctx.check(self.lib.numa_gpu_hmg2d_levels(self.h, C.byref(v)), "hmg2d_levels")
        return v.value

    def __call__(self, r: Vec, z: Vec):
        self.ctx.check(self.lib.numa_gpu_hmg2d_apply(self.h, r.h, z.h), "hmg2d_apply")


class LearnedNet:
    """The learned preconditioner's network (include/numa_gpu.h, numa_gpu_learned_*)."""

    def __init__(self, ctx: Context, n0: int = 31, seed: int = 1):
        self.ctx, self.lib, self.n0 = ctx, ctx.lib, int(n0)
        h = C.c_void_p()
        ctx.check(self.lib.numa_gpu_learned_create(ctx.h, self.n0, seed, C.byref(h)), "learned_create")
        self.h = h
        self.ctx._adopt(self)

    def close(self):
        if self.h and _ctx_open(self.ctx):
            self.lib.numa_gpu_learned_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def num_params(self) -> int:
        v = C.c_size_t()
        self.ctx.check(self.lib.numa_gpu_learned_num_params(self.h, C.byref(v)), "learned_num_params")
        return v.value

    def get_params(self) -> np.ndarray:
        p = np.empty(self.num_params(), dtype=np.float32)
        self.ctx.check(self.lib.numa_gpu_learned_get_params(self.h, p.ctypes.data_as(_F32P), p.size), "get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self.ctx.check(self.lib.numa_gpu_learned_set_params(self.h, p.ctypes.data_as(_F32P), p.size), "set_params")

    def forward(self, features) -> np.ndarray:
        f = np.ascontiguousarray(features, dtype=np.float32)
        out = np.empty(self.n0 ** 3, dtype=np.float32)
        self.ctx.check(self.lib.numa_gpu_learned_forward(self.h, f.ctypes.data_as(_F32P), out.ctypes.data_as(_F32P)),
                       "learned_forward")
        return out

    def train(self, n_fine: int, instances: int = 8, states: int = 3, rhs_per_state: int = 8,
              krylov_per_state: int = 4, epochs: int = 4, batch: int = 8, lr: float = 1e-3, lambda_min: float = 1.0,
              lambda_max: float = 6.5, seed: int = 7, solve_rtol: float = 1e-6) -> dict:
        """Generates residual-error pairs on the GPU and trains (numa_gpu_learned_train)."""
        p = LearnedTrainParams(n_fine, lambda_min, lambda_max, instances, states, rhs_per_state, krylov_per_state,
                               epochs, batch, lr, seed, solve_rtol)
        rep = LearnedTrainReport()
        self.ctx.check(self.lib.numa_gpu_learned_train(self.h, C.byref(p), C.byref(rep)), "learned_train")
        return to_dict(rep)

    def gradient(self, features, target):
        f = np.ascontiguousarray(features, dtype=np.float32)
        t = np.ascontiguousarray(target, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        g = np.empty(self.num_params(), dtype=np.float32)
        self.ctx.check(self.lib.numa_gpu_learned_gradient(self.h, f.ctypes.data_as(_F32P), t.ctypes.data_as(_F32P),
                                                          loss.ctypes.data_as(_F32P), g.ctypes.data_as(_F32P)),
                       "learned_gradient")
        return float(loss[0]), g


class PoissonMG:
    """PoissonMG(n, pre, post) (linalg/poisson_mg.hpp:24-64); precision / max_levels extend it."""

    def __init__(self, ctx: Context, n: int, pre: int = 2, post: int = 2, precision: int = FP64,
                 max_levels: int = 0):
        self.ctx, self.lib, self.n = ctx, ctx.lib, int(n)
        h = C.c_void_p()
        ctx.check(self.lib.numa_gpu_mg_create_ex(ctx.h, self.n, pre, post, precision, max_levels, C.byref(h)),
                  "mg_create")
        self.h = h
        self.ctx._adopt(self)

    def close(self):
        if self.h and _ctx_open(self.ctx):
            self.lib.numa_gpu_mg_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def levels(self) -> int:
        v = C.c_size_t()
        self.ctx.check(self.lib.numa_gpu_mg_levels(self.h, C.byref(v)), "mg_levels")
        return v.value

    def time_smoother(self, reps: int = 20) -> float:
        """Average ms of one finest-level colour pass (diagnostic)."""
        v = C.c_double()
        self.ctx.check(self.lib.numa_gpu_diag_time_smoother(self.h, reps, C.byref(v)), "diag_time_smoother")
        return v.value

    def __call__(self, r: Vec, z: Vec):
        self.ctx.check(self.lib.numa_gpu_mg_apply(self.h, r.h, z.h), "mg_apply")


class Provider:
    """A preconditioner provider: make(x) binds it, apply(r, z) applies it."""

    def __init__(self, ctx: Context, handle, kind: str):
        self.ctx, self.lib, self.h, self.kind = ctx, ctx.lib, handle, kind
        ctx._adopt(self)

    @classmethod
    def identity(cls, ctx: Context) -> "Provider":
        h = C.c_void_p()
        ctx.check(ctx.lib.numa_gpu_provider_create_identity(ctx.h, C.byref(h)), "provider_identity")
        return cls(ctx, h, "none")

    @classmethod
    def poisson_mg(cls, ctx: Context, n: int, pre: int = 2, post: int = 2, precision: int = FP64) -> "Provider":
        h = C.c_void_p()
        ctx.check(ctx.lib.numa_gpu_provider_create_poisson_mg(ctx.h, n, pre, post, precision, C.byref(h)),
                  "provider_poisson_mg")
        return cls(ctx, h, "mg")

    @classmethod
    def jacobian_mg(cls, ctx: Context, n: int, pre: int = 2, post: int = 2) -> "Provider":
        """The FP32 V-cycle with Jacobian-aware coarse levels (n <= 15 solve with -Lap_h - lambda e^u)."""
        h = C.c_void_p()
        ctx.check(ctx.lib.numa_gpu_provider_create_jacobian_mg(ctx.h, n, pre, post, C.byref(h)),
                  "provider_jacobian_mg")
        return cls(ctx, h, "jacobian_mg")

    @classmethod
    def jacobi(cls, op: Bratu3D) -> "Provider":
        h = C.c_void_p()
        op.ctx.check(op.lib.numa_gpu_provider_create_jacobi(op.h, C.byref(h)), "provider_jacobi")
        p = cls(op.ctx, h, "jacobi")
        p._op = op  # keep the operator alive
        return p

    @classmethod
    def burgers_mg(cls, ctx: Context, n: int, nu: float, dt: float) -> "Provider":
        """BurgersMGProvider(n, nu, dt) (problems/burgers2d.hpp:220-246)."""
        h = C.c_void_p()
        ctx.check(ctx.lib.numa_gpu_provider_create_burgers_mg(ctx.h, n, nu, dt, C.byref(h)), "provider_burgers_mg")
        return cls(ctx, h, "burgers_mg")

    @classmethod
    def brusselator_jacobi(cls, op: "Brusselator1D") -> "Provider":
        """BrusselatorJacobi{op} (problems/brusselator1d.hpp:194-222)."""
        h = C.c_void_p()
        op.ctx.check(op.lib.numa_gpu_provider_create_brusselator_jacobi(op.h, C.byref(h)), "provider_bruss_jacobi")
        p = cls(op.ctx, h, "bruss_jacobi")
        p._op = op
        return p

    @classmethod
    def brusselator_mg(cls, op: "Brusselator2D", precision: int = FP64, pre: int = 2, post: int = 2) -> "Provider":
        """The coupled-block periodic multigrid, bound at each Newton iterate."""
        h = C.c_void_p()
        op.ctx.check(op.lib.numa_gpu_provider_create_brusselator_mg(op.h, precision, pre, post, C.byref(h)),
                     "provider_bruss_mg")
        p = cls(op.ctx, h, "bruss_mg")
        p._op = op
        return p

    @classmethod
    def learned(cls, ctx: Context, n: int, net: "LearnedNet", stall: float = 0.9) -> "Provider":
        """FP32 V-cycle + learned coarse correction (for FGMRES)."""
        h = C.c_void_p()
        ctx.check(ctx.lib.numa_gpu_provider_create_learned(ctx.h, n, net.h, stall, C.byref(h)), "provider_learned")
        p = cls(ctx, h, "learned")
        p._net = net
        return p

    def learned_stats(self) -> tuple[int, int]:
        a, f = C.c_size_t(), C.c_size_t()
        self.ctx.check(self.lib.numa_gpu_provider_learned_stats(self.h, C.byref(a), C.byref(f)), "learned_stats")
        return a.value, f.value

    @classmethod
    def create(cls, ctx: Context, kind: str, op, precision: int = FP64) -> "Provider | None":
        if isinstance(op, Burgers2D):
            return cls.burgers_mg(ctx, op.n, op.nu, op.dt) if kind == "mg" else cls.identity(ctx)
        if isinstance(op, Brusselator1D):
            return cls.brusselator_jacobi(op) if kind == "jacobi" else cls.identity(ctx)
        if isinstance(op, Brusselator2D):
            return cls.brusselator_mg(op, precision) if kind == "mg" else cls.identity(ctx)
        if kind == "mg":
            return cls.poisson_mg(ctx, op.n, precision=precision)
        if kind == "jacobi":
            return cls.jacobi(op)
        return cls.identity(ctx)

    def close(self):
        if self.h and _ctx_open(self.ctx):
            self.lib.numa_gpu_provider_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def make(self, x: Vec):
        self.ctx.check(self.lib.numa_gpu_provider_make(self.h, x.h), "provider_make")
        return self

    def apply(self, r: Vec, z: Vec):
        self.ctx.check(self.lib.numa_gpu_provider_apply(self.h, r.h, z.h), "provider_apply")


class KrylovSpace:
    """Saved Arnoldi basis (linalg/gmres.hpp:25-35), on the device."""

    def __init__(self, ctx: Context):
        self.ctx, self.lib = ctx, ctx.lib
        h = C.c_void_p()
        ctx.check(self.lib.numa_gpu_krylov_space_create(ctx.h, C.byref(h)), "krylov_space_create")
        self.h = h
        self.ctx._adopt(self)

    def close(self):
        if self.h and _ctx_open(self.ctx):
            self.lib.numa_gpu_krylov_space_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def k(self) -> int:
        v = C.c_size_t()
        self.ctx.check(self.lib.numa_gpu_krylov_space_k(self.h, C.byref(v)), "krylov_space_k")
        return v.value


def gmres(ctx: Context, apply, b: Vec, x: Vec, rtol: float, restart: int, max_iters: int, precond=None,
          zero_guess: bool = True, orth: int = MGS, flexible: bool = False, save: KrylovSpace | None = None,
          r_init: Vec | None = None) -> dict:
    """gmres(apply, precond, b, x, ...) (linalg/gmres.hpp:61-65) with Python callables
    apply(v: Vec, out: Vec) and precond(r: Vec, z: Vec) on device vectors."""
    errors = []

    def _wrap(fn):
        def cb(user, vp, op):
            try:
                fn(Vec(ctx, b.n, vp), Vec(ctx, b.n, op))
                return 0
            except Exception as e:  # reported through the status code
                errors.append(e)
                return 1
        return cb

    a_cb = APPLY_FN(_wrap(apply))
    p_cb = PRECOND_FN(_wrap(precond)) if precond is not None else PRECOND_FN()
    res = GmresResult()
    rc = ctx.lib.numa_gpu_gmres(ctx.h, a_cb, None, p_cb, None, b.h, x.h, rtol, restart, max_iters,
                                int(zero_guess), orth, int(flexible), save.h if save else None,
                                r_init.h if r_init else None, C.byref(res))
    if errors:
        raise errors[0]
    ctx.check(rc, "gmres")
    return to_dict(res)


def gmres_bratu3d(op: Bratu3D, xpt: Vec, b: Vec, x: Vec, rtol: float, restart: int, max_iters: int,
                  provider: Provider | None = None, jvp_mode: int = ANALYTIC, zero_guess: bool = True,
                  orth: int = MGS, flexible: bool = False, save: KrylovSpace | None = None,
                  r_init: Vec | None = None) -> dict:
    res = GmresResult()
    op.ctx.check(op.lib.numa_gpu_gmres_bratu3d(op.h, xpt.h, jvp_mode, provider.h if provider else None, b.h, x.h,
                                               rtol, restart, max_iters, int(zero_guess), orth, int(flexible),
                                               save.h if save else None, r_init.h if r_init else None,
                                               C.byref(res)), "gmres_bratu3d")
    return to_dict(res)


def gmres_recycled_bratu3d(op: Bratu3D, xpt: Vec, b: Vec, x: Vec, rtol: float, restart: int, max_iters: int,
                           space: KrylovSpace, provider: Provider | None = None, jvp_mode: int = ANALYTIC,
                           orth: int = MGS, save: KrylovSpace | None = None) -> dict:
    res = GmresResult()
    op.ctx.check(op.lib.numa_gpu_gmres_recycled_bratu3d(op.h, xpt.h, jvp_mode, provider.h if provider else None,
                                                        b.h, x.h, rtol, restart, max_iters, orth, space.h,
                                                        save.h if save else None, C.byref(res)),
                 "gmres_recycled_bratu3d")
    return to_dict(res)


def mg_apply_noalloc(n: int, r: Vec, z: Vec, pre: int = 2, post: int = 2, stream: int | None = None) -> int:
    """One FP64 V-cycle with no device allocation (numa_gpu_mg_apply_noalloc): for callers that
    cannot allocate device memory when they apply the preconditioner.  Grids up to 63^3; work
    arrays in a fixed 4.8 MB static device array shared by all calls (order calls on one
    stream).  Enqueues on `stream` (default: the vectors' context stream) and returns the
    status code without waiting."""
    s = r.ctx.stream() if stream is None else stream
    return r.lib.numa_gpu_mg_apply_noalloc(n, pre, post, C.c_void_p(r.device_ptr()), C.c_void_p(z.device_ptr()),
                                          C.c_void_p(s))


def diag_exp(x: "Vec", out: "Vec", cuda_ref: "Vec | None" = None):
    """out = the library's FP64 e^x (table-driven, as in the residual kernels); cuda_ref = CUDA's exp."""
    x.ctx.check(x.lib.numa_gpu_diag_exp(x.h, out.h, cuda_ref.h if cuda_ref is not None else None), "diag_exp")


def diag_div(a: "Vec", b: float, out: "Vec"):
    """out = a / b through the finite-difference quotients' reciprocal form (correctly rounded)."""
    a.ctx.check(a.lib.numa_gpu_diag_div(a.h, float(b), out.h), "diag_div")


def diag_conv3d(ctx: Context, n: int, x: np.ndarray, w: np.ndarray, bias: np.ndarray | None = None,
                adjoint: bool = False) -> np.ndarray:
    """One tensor-core 3x3x3 convolution (BF16 operands, FP32 accumulation), host arrays in and out.
    x: [n^3, cin] (adjoint: [n^3, cout]), w: [27, cin, cout]; returns [n^3, cout] (adjoint: [n^3, cin])."""
    w = np.ascontiguousarray(w, dtype=np.float32)
    cin, cout = int(w.shape[1]), int(w.shape[2])
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty((n ** 3, cin if adjoint else cout), dtype=np.float32)
    b = None if bias is None else np.ascontiguousarray(bias, dtype=np.float32)
    rc = ctx.lib.numa_gpu_diag_conv3d(ctx.h, n, cin, cout, 1 if adjoint else 0, x.ctypes.data_as(_F32P),
                                      w.ctypes.data_as(_F32P), None if b is None else b.ctypes.data_as(_F32P),
                                      y.ctypes.data_as(_F32P))
    ctx.check(rc, "diag_conv3d")
    return y


def diag_conv3d_wgrad(ctx: Context, n: int, x: np.ndarray, g: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """The tensor-core weight and bias gradients of one 3x3x3 convolution: x [n^3, cin], g [n^3, cout];
    returns dw [27, cin, cout] and db [cout]."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    g = np.ascontiguousarray(g, dtype=np.float32)
    cin, cout = int(x.shape[1]), int(g.shape[1])
    dw = np.empty((27, cin, cout), dtype=np.float32)
    db = np.empty(cout, dtype=np.float32)
    rc = ctx.lib.numa_gpu_diag_conv3d_wgrad(ctx.h, n, cin, cout, x.ctypes.data_as(_F32P), g.ctypes.data_as(_F32P),
                                            dw.ctypes.data_as(_F32P), db.ctypes.data_as(_F32P))
    ctx.check(rc, "diag_conv3d_wgrad")
    return dw, db


def forcing(params: KrylovParams, k: int, rnorm: float, rprev: float, eta_prev: float, res0: float) -> float:
    return load().numa_gpu_forcing(C.byref(params), k, rnorm, rprev, eta_prev, res0)


_DRIVER_METHOD = {"numa_gpu_newton_krylov": 0, "numa_gpu_chebyshev_inexact": 1, "numa_gpu_tf_chebyshev_2018": 3}


def _driver(name: str, op, x: Vec, params: KrylovParams | None, provider: Provider | None) -> dict:
    p = params if params is not None else default_params()
    res = KrylovResult()
    if isinstance(op, Burgers2D):
        rc = op.lib.numa_gpu_burgers2d_solve(op.h, _DRIVER_METHOD[name], x.h, C.byref(p),
                                             provider.h if provider else None, C.byref(res))
    elif isinstance(op, (Brusselator1D, Brusselator2D)):
        fn = "numa_gpu_brusselator1d_solve" if isinstance(op, Brusselator1D) else "numa_gpu_brusselator2d_solve"
        rc = getattr(op.lib, fn)(op.h, _DRIVER_METHOD[name], x.h, C.byref(p), provider.h if provider else None,
                                 C.byref(res))
    else:
        rc = getattr(op.lib, name)(op.h, x.h, C.byref(p), provider.h if provider else None, C.byref(res))
    op.ctx.check(rc, name)
    return to_dict(res)


def newton_krylov(op: Bratu3D, x: Vec, params: KrylovParams | None = None, provider: Provider | None = None) -> dict:
    """newton_krylov (methods/krylov_newton.hpp:69-114); x: x0 in, solution out."""
    return _driver("numa_gpu_newton_krylov", op, x, params, provider)


def chebyshev_inexact(op: Bratu3D, x: Vec, params: KrylovParams | None = None,
                      provider: Provider | None = None) -> dict:
    """chebyshev_inexact (methods/krylov_newton.hpp:116-189)."""
    return _driver("numa_gpu_chebyshev_inexact", op, x, params, provider)


def tf_chebyshev_2018(op: Bratu3D, x: Vec, params: KrylovParams | None = None,
                      provider: Provider | None = None) -> dict:
    """tf_chebyshev_2018 (methods/tf_chebyshev_2018.hpp:52-132)."""
    return _driver("numa_gpu_tf_chebyshev_2018", op, x, params, provider)


def solve(op: Bratu3D, x: Vec, method: str = "nk", params: KrylovParams | None = None,
          provider: Provider | None = None) -> dict:
    p = params if params is not None else default_params()
    if method == "rec":
        p.recycle = 1
        return chebyshev_inexact(op, x, p, provider)
    return {"nk": newton_krylov, "cheb": chebyshev_inexact, "tf2018": tf_chebyshev_2018}[method](op, x, p, provider)


def solve_bratu3d_host(ctx: Context, n: int, lam: float, x0: np.ndarray, out: np.ndarray | None = None,
                       method: str = "nk", precond: str = "mg", mg_precision: int = FP64,
                       params: KrylovParams | None = None) -> tuple[np.ndarray, dict]:
    """Host buffers in, host buffers out (numa_gpu_solve_bratu3d_host)."""
    p = params if params is not None else default_params()
    x0 = _f64(x0).ravel()
    if out is None:
        out = np.empty(n ** 3)
    res = KrylovResult()
    rc = ctx.lib.numa_gpu_solve_bratu3d_host(ctx.h, n, lam, METHODS[method], PRECONDS[precond], mg_precision,
                                             C.byref(p), x0.ctypes.data_as(_F64P), out.ctypes.data_as(_F64P),
                                             C.byref(res))
    ctx.check(rc, "solve_bratu3d_host")
    return out, to_dict(res)


def solve_burgers2d_host(ctx: Context, n: int, nu: float, dt: float, amplitude: float, x0: np.ndarray,
                         out: np.ndarray | None = None, method: str = "nk", precond: str = "mg",
                         params: KrylovParams | None = None) -> tuple[np.ndarray, dict]:
    """Host buffers in, host buffers out (numa_gpu_solve_burgers2d_host); precond "mg" or "none"."""
    p = params if params is not None else default_params()
    x0 = _f64(x0).ravel()
    if out is None:
        out = np.empty(2 * n * n)
    res = KrylovResult()
    kind = PRECONDS["burgers_mg"] if precond == "mg" else PRECONDS["none"]
    rc = ctx.lib.numa_gpu_solve_burgers2d_host(ctx.h, n, nu, dt, amplitude, METHODS[method], kind, C.byref(p),
                                               x0.ctypes.data_as(_F64P), out.ctypes.data_as(_F64P), C.byref(res))
    ctx.check(rc, "solve_burgers2d_host")
    return out, to_dict(res)


def solve_brusselator1d_host(ctx: Context, n: int, dt: float, x0: np.ndarray | None = None, method: str = "nk",
                             precond: str = "jacobi", params: KrylovParams | None = None) -> tuple[np.ndarray, dict]:
    """Host buffers (numa_gpu_solve_brusselator1d_host); x0 None: the previous state; precond "jacobi" or "none"."""
    p = params if params is not None else default_params()
    out = np.empty(2 * n)
    res = KrylovResult()
    kind = PRECONDS["bruss_jacobi"] if precond == "jacobi" else PRECONDS["none"]
    keep = None if x0 is None else _f64(x0).ravel()
    x0p = None if keep is None else keep.ctypes.data_as(_F64P)
    rc = ctx.lib.numa_gpu_solve_brusselator1d_host(ctx.h, n, dt, METHODS[method], kind, C.byref(p), x0p,
                                                   out.ctypes.data_as(_F64P), C.byref(res))
    ctx.check(rc, "solve_brusselator1d_host")
    return out, to_dict(res)


def brusselator2d_advance_host(ctx: Context, n: int, x0: np.ndarray, steps: int, params: BrusselatorParams | None = None,
                               method: str = "nk", precond: str = "mg", mg_precision: int = FP32,
                               kparams: KrylovParams | None = None, out: np.ndarray | None = None
                               ) -> tuple[np.ndarray, list[dict]]:
    """Host buffers (numa_gpu_brusselator2d_advance_host): `steps` implicit-Euler steps from x0."""
    prm = params if params is not None else brusselator_params()
    p = kparams if kparams is not None else default_params()
    if method == "rec":
        p.recycle = 1
    x0 = _f64(x0).ravel()
    if out is None:
        out = np.empty(2 * n * n)
    res = (KrylovResult * steps)()
    kind = PRECONDS["bruss_mg"] if precond == "mg" else PRECONDS["none"]
    rc = ctx.lib.numa_gpu_brusselator2d_advance_host(ctx.h, n, C.byref(prm), steps, METHODS[method], kind,
                                                     mg_precision, C.byref(p), x0.ctypes.data_as(_F64P),
                                                     out.ctypes.data_as(_F64P), res)
    ctx.check(rc, "brusselator2d_advance_host")
    return out, [to_dict(r) for r in res]


def solve_batch(instances, method: str = "nk", mg_precision: int = FP32, params: KrylovParams | None = None,
                workers: int = 16, device: int = 0) -> tuple[list[dict], float]:
    """numa_gpu_solve_batch: instances = [(n, lambda), ...]; returns per-instance results and wall seconds."""
    lib = load()
    arr = (BatchInstance * len(instances))(*[BatchInstance(int(n), float(lam)) for n, lam in instances])
    res = (BatchResult * len(instances))()
    wall = C.c_double()
    p = params if params is not None else default_params()
    rc = lib.numa_gpu_solve_batch(device, arr, len(instances), METHODS[method], mg_precision, C.byref(p), workers, res,
                                  C.byref(wall))
    if rc != OK:
        raise NumaGPUError(rc, "numa_gpu_solve_batch", lib.numa_gpu_batch_last_error().decode())
    return [to_dict(r) for r in res], wall.value


class BatchExecutor:
    """numa_gpu_batch_*: worker contexts and solvers kept between batches."""

    def __init__(self, workers: int = 16, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.numa_gpu_batch_create(device, workers, C.byref(h))
        if rc != OK:
            raise NumaGPUError(rc, "numa_gpu_batch_create", self.lib.numa_gpu_batch_last_error().decode())
        self.h = h
        _live_contexts.add(self)  # closed at exit like a context (it owns worker contexts)

    def close(self):
        if self.h:
            self.lib.numa_gpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_workers(self, workers: int):
        rc = self.lib.numa_gpu_batch_set_workers(self.h, workers)
        if rc != OK:
            raise NumaGPUError(rc, "numa_gpu_batch_set_workers", self.lib.numa_gpu_batch_last_error().decode())

    def autotune(self, instances, candidates=(4, 8, 16, 24, 32), method: str = "nk", mg_precision: int = FP32,
                 params: KrylovParams | None = None) -> tuple[int, dict]:
        """Picks the worker count (the schedule) that runs these instances fastest; returns it and the
        seconds of every candidate."""
        arr = (BatchInstance * len(instances))(*[BatchInstance(int(n), float(lam)) for n, lam in instances])
        cand = (C.c_int * len(candidates))(*candidates)
        secs = (C.c_double * len(candidates))()
        chosen = C.c_int()
        p = params if params is not None else default_params()
        rc = self.lib.numa_gpu_batch_autotune(self.h, arr, len(instances), METHODS[method], mg_precision, C.byref(p),
                                              cand, len(candidates), C.byref(chosen), secs)
        if rc != OK:
            raise NumaGPUError(rc, "numa_gpu_batch_autotune", self.lib.numa_gpu_batch_last_error().decode())
        return chosen.value, {int(c): float(t) for c, t in zip(candidates, secs)}

    def solve(self, instances, method: str = "nk", mg_precision: int = FP32,
              params: KrylovParams | None = None) -> tuple[list[dict], float]:
        arr = (BatchInstance * len(instances))(*[BatchInstance(int(n), float(lam)) for n, lam in instances])
        res = (BatchResult * len(instances))()
        wall = C.c_double()
        p = params if params is not None else default_params()
        rc = self.lib.numa_gpu_batch_solve(self.h, arr, len(instances), METHODS[method], mg_precision, C.byref(p),
                                           res, C.byref(wall))
        if rc != OK:
            raise NumaGPUError(rc, "numa_gpu_batch_solve", self.lib.numa_gpu_batch_last_error().decode())
        return [to_dict(r) for r in res], wall.value


class BatchSolver:
    """numa_gpu_bsolver_*: many Bratu3D instances (n = 2^k - 1, 31 ... 1023) solved together by the
    mixed Newton-Krylov path, one launch per operation over all of them, scalar decisions on the
    device, Arnoldi steps and line-search trials as captured CUDA graphs."""

    def __init__(self, ctx: Context, instances, params: KrylovParams | None = None):
        self.ctx, self.lib = ctx, ctx.lib
        self.instances = [(int(n), float(lam)) for n, lam in instances]
        arr = (BatchInstance * len(self.instances))(*[BatchInstance(n, lam) for n, lam in self.instances])
        p = params if params is not None else default_params()
        h = C.c_void_p()
        ctx.check(self.lib.numa_gpu_bsolver_create(ctx.h, arr, len(self.instances), C.byref(p), C.byref(h)),
                  "bsolver_create")
        self.h = h
        ctx._adopt(self)

    def close(self):
        if self.h and _ctx_open(self.ctx):
            self.lib.numa_gpu_bsolver_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, want_x: bool = False):
        """Returns (per-instance result dicts, seconds, solutions or None) in the order given."""
        res = (BatchResult * len(self.instances))()
        secs = C.c_double()
        x = None
        if want_x:
            x = np.empty(sum(n ** 3 for n, _ in self.instances))
        self.ctx.check(self.lib.numa_gpu_bsolver_solve(self.h, x.ctypes.data_as(_F64P) if x is not None else None, res,
                                                       C.byref(secs)), "bsolver_solve")
        xs = None
        if x is not None:
            xs, o = [], 0
            for n, _ in self.instances:
                xs.append(x[o:o + n ** 3])
                o += n ** 3
        return [to_dict(r) for r in res], secs.value, xs

    def tuning(self) -> dict:
        t = BatchTuning()
        self.ctx.check(self.lib.numa_gpu_bsolver_get_tuning(self.h, C.byref(t)), "bsolver_get_tuning")
        return {"planes": t.planes, "elems_per_block": t.elems_per_block}

    def set_tuning(self, planes: int, elems_per_block: int):
        t = BatchTuning(planes, elems_per_block)
        self.ctx.check(self.lib.numa_gpu_bsolver_set_tuning(self.h, C.byref(t)), "bsolver_set_tuning")

    def autotune(self, planes=(2, 4, 8), elems=(8192, 16384, 32768), cache: str | Path | None = None) -> dict:
        """Picks the fastest tile shapes on this batch (one warm and one timed batch per candidate); with
        `cache`, a JSON file of earlier choices keyed by the batch's size histogram is read first and
        updated after tuning."""
        import json
        key = None
        if cache is not None:
            hist = {}
            for n, _ in self.instances:
                hist[n] = hist.get(n, 0) + 1
            key = ",".join(f"{n}x{c}" for n, c in sorted(hist.items()))
            path = Path(cache)
            book = json.loads(path.read_text()) if path.exists() else {}
            if key in book:
                self.set_tuning(book[key]["planes"], book[key]["elems_per_block"])
                return dict(book[key], cached=True)
        pa = (C.c_int * len(planes))(*planes)
        ea = (C.c_int * len(elems))(*elems)
        secs = (C.c_double * (len(planes) * len(elems)))()
        t = BatchTuning()
        self.ctx.check(self.lib.numa_gpu_bsolver_autotune(self.h, pa, len(planes), ea, len(elems), C.byref(t), secs),
                       "bsolver_autotune")
        out = {"planes": t.planes, "elems_per_block": t.elems_per_block,
               "seconds": {f"{p}x{e}": float(secs[a * len(elems) + b]) for a, p in enumerate(planes)
                           for b, e in enumerate(elems)}}
        if key is not None:
            book[key] = {"planes": t.planes, "elems_per_block": t.elems_per_block}
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(book, indent=1))
        return out
