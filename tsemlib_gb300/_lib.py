"""ctypes binding of libtsemgpu.so (the C ABI in include/tsem_gpu.h).

The library is built in-tree by tsemlib_gb300.build; loading fails loudly when it
is missing -- there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

# TSEM_LIB_VARIANT=check loads the checked build (bounds checks, see build.py)
VARIANT = os.environ.get("TSEM_LIB_VARIANT") or None
LIB_PATH = _build.lib_path(VARIANT)

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double

STATUS = {0: "OK", 1: "MAXIT", 2: "BREAKDOWN", 3: "NONFINITE", 4: "OOM_REFUSED", 5: "TIMEOUT", 6: "INVALID",
          7: "CUDA_ERROR", 8: "NO_DEVICE"}


class TsemError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Mesh(ctypes.Structure):
    _fields_ = [("nv", _I32), ("ne", _I32), ("nf", _I32), ("nt", _I32),
                ("xyz", _P), ("edge_v", _P), ("face_v", _P), ("face_e", _P), ("tet_v", _P), ("tet_f", _P),
                ("mark_v", _P), ("mark_e", _P), ("mark_f", _P), ("femdof_v", _P), ("femdof_e", _P)]


class SolverOpts(ctypes.Structure):
    _fields_ = [("precond", _I32), ("pmg_order_step", _I32), ("smooth_steps", _I32), ("smoother", _I32),
                ("tol_abs_l1", _D), ("tol_rel", _D), ("max_iter", _I32), ("inner_tol", _D), ("omega", _D)]


class Stats(ctypes.Structure):
    _fields_ = [("iterations", _I32), ("status", _I32), ("residual_l1", _D), ("init_l1", _D),
                ("residual_rel", _D), ("device_ms", _D)]

    def as_dict(self):
        return dict(iterations=self.iterations, status=STATUS.get(self.status, self.status),
                    residual_l1=self.residual_l1, init_l1=self.init_l1, residual_rel=self.residual_rel,
                    device_ms=self.device_ms)


class Request(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int64), ("kind", ctypes.c_int32), ("n_cube", ctypes.c_int32),
                ("order", ctypes.c_int32), ("n_eig", ctypes.c_int32), ("jitter", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("tol", ctypes.c_double), ("tol_eig", ctypes.c_double),
                ("arrival_s", ctypes.c_double), ("x_out", ctypes.c_void_p)]


class Result(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int64), ("status", ctypes.c_int32), ("iterations", ctypes.c_int32),
                ("n_dof", ctypes.c_int64), ("queued_s", ctypes.c_double), ("latency_s", ctypes.c_double),
                ("finish_s", ctypes.c_double), ("setup_s", ctypes.c_double), ("solve_s", ctypes.c_double),
                ("residual", ctypes.c_double), ("checksum", ctypes.c_double), ("norm2", ctypes.c_double),
                ("lambda0", ctypes.c_double), ("lambda_last", ctypes.c_double)]

    def as_dict(self):
        d = {name: getattr(self, name) for name, _ in self._fields_}
        d["status"] = STATUS.get(self.status, self.status)
        return d


class ServeOpts(ctypes.Structure):
    _fields_ = [("workers", ctypes.c_int32), ("plain", ctypes.c_int32), ("realtime", ctypes.c_int32),
                ("memory_budget_bytes", ctypes.c_double)]


SIGNATURES = {
    "tsem_last_error": (ctypes.c_char_p, []),
    "tsem_kernel_launches": (ctypes.c_int64, []),
    "tsem_debug_wait_limit": (_I32, [ctypes.c_int64]),
    "tsem_debug_bounds": (_I32, [_I32, _P, _P, _P]),
    "tsem_solve_batch": (_I32, [_P, _I32, _P, _P, _I32, _P, _P]),
    "tsem_batch_create": (_I32, [_P, _P]),
    "tsem_batch_destroy": (None, [_P]),
    "tsem_batch_submit": (_I32, [_P, _P, _P, _P, _P]),
    "tsem_batch_poll": (_I32, [_P, _I32, _P, _P, _P, _P]),
    "tsem_batch_cancel": (_I32, [_P, ctypes.c_int64]),
    "tsem_space_create": (_I32, [ctypes.POINTER(Mesh), _I32, _I32, ctypes.POINTER(_P)]),
    "tsem_space_set_quadrature": (_I32, [_P, _I32, _P, _P, _I32, _P, _P, _I32, _P, _P]),
    "tsem_space_destroy": (None, [_P]),
    "tsem_space_info": (_I32, [_P, _P]),
    "tsem_space_numbering": (_I32, [_P, _P, _P]),
    "tsem_space_transform": (_I32, [_P, _P, _P, _P]),
    "tsem_space_geometry": (_I32, [_P] * 9),
    "tsem_space_sum_dof": (_I32, [_P, _P]),
    "tsem_space_quadrature": (_I32, [_P] * 7),
    "tsem_element_qpoints": (_I32, [_P, _P]),
    "tsem_boundary_points": (_I32, [_P, _I32, _P, ctypes.POINTER(_I64)]),
    "tsem_geometry_marks": (_I32, [_P, _I32, _P, ctypes.POINTER(_I64)]),
    "tsem_multiindex": (_I32, [_I32, _P, _P]),
    "tsem_face_table": (_I32, [_I32, ctypes.POINTER(_I64), _P, _P, _P, _P, _P, _P]),
    "tsem_reference_matrix": (_I32, [_P, _I32, _P, _P]),
    "tsem_assemble": (_I32, [_P, _I32, ctypes.POINTER(_P)]),
    "tsem_csr_info": (_I32, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "tsem_csr_export": (_I32, [_P, _P, _P, _P]),
    "tsem_csr_import": (_I32, [_I64, _P, _P, _P, ctypes.POINTER(_P)]),
    "tsem_csr_copy": (_I32, [_P, ctypes.POINTER(_P)]),
    "tsem_csr_destroy": (None, [_P]),
    "tsem_csr_spmv": (_I32, [_P, _P, _P, _I32, _P]),
    "tsem_csr_spmv_tuning": (_I32, [_P, _P, _P, _P, _P, _I32, _P]),
    "tsem_rhs": (_I32, [_P, _P, _P]),
    "tsem_neumann": (_I32, [_P, _P, _P, _I32]),
    "tsem_dirichlet": (_I32, [_P, _P, _P, _P, _P, _P, _I32, _I32]),
    "tsem_zero_bc": (_I32, [_P, _P, _P, _I32]),
    "tsem_errors": (_I32, [_P, _P, _P, _P, _P]),
    "tsem_solver_create": (_I32, [_P, _P, _I32, ctypes.POINTER(SolverOpts), ctypes.POINTER(_P)]),
    "tsem_solver_destroy": (None, [_P]),
    "tsem_solve_pcg": (_I32, [_P, _P, _P, ctypes.POINTER(Stats)]),
    "tsem_solve_pcg_device": (_I32, [_P, _P, _P, ctypes.POINTER(Stats), _P]),
    "tsem_solve_pmg": (_I32, [_P, _P, _P, ctypes.c_double, _I32, ctypes.POINTER(Stats)]),
    "tsem_solve_lobpcg": (_I32, [_P, _P, _I32, _I32, _P, _P, ctypes.c_double, _I32, ctypes.POINTER(Stats)]),
    "tsem_solve_lobpcg_pencil": (_I32, [_P, _P, _P, _I32, _I32, _P, _P, ctypes.c_double, _I32, ctypes.POINTER(Stats)]),
    "tsem_solve_lobpcg_device": (_I32, [_P, _P, _I32, _I32, _P, _P, ctypes.c_double, _I32, ctypes.POINTER(Stats), _P]),
    "tsem_pmg_vcycle": (_I32, [_P, _P, _P]),
    "tsem_solver_create_mixed": (_I32, [_P, _P, _I32, ctypes.POINTER(SolverOpts), ctypes.POINTER(_P)]),
    "tsem_mf_apply": (_I32, [_P, _I32, _I32, _P, _P, ctypes.POINTER(_I64)]),
    "tsem_mf_apply_device": (_I32, [_P, _I32, _I32, _P, _P, _P]),
    "tsem_mf_apply_device_noalloc": (_I32, [_P, _I32, _P, _P, _P]),
    "tsem_mf_profile": (_I32, [_P, _I32, _I32, _I32, _P]),
    "tsem_mf_vcycle_device": (_I32, [_P, _I32, _P, _P, _P]),
    "tsem_assemble_potential": (_I32, [_P, _P, ctypes.POINTER(_P)]),
    "tsem_eval_qp": (_I32, [_P, _P, _P]),
    "tsem_eval_qp_device": (_I32, [_P, _P, _P, _P]),
    "tsem_density": (_I32, [_P, _P, _I32, _P, _P]),
    "tsem_density_device": (_I32, [_P, _P, _I32, _P, _P, _P]),
    "tsem_density_l2_difference": (_I32, [_P, _P, _P, _I32, _P, _P]),
    "tsem_rhs_device": (_I32, [_P, _P, _P, _P]),
    "tsem_assemble_potential_device": (_I32, [_P, _P, ctypes.POINTER(_P), _P]),
    "tsem_interpolation": (_I32, [_P, _P, _P, _P, _P, _P]),
    "tsem_csr_add": (_I32, [_P, ctypes.c_double, _P]),
    "tsem_serve": (_I32, [ctypes.POINTER(Request), ctypes.c_int64, ctypes.POINTER(ServeOpts), ctypes.POINTER(Result)]),
}

_lib = None


def lib(build_if_missing: bool = True):
    """Load libtsemgpu.so, building it first when it is absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise OSError(f"{LIB_PATH} is missing; run `python -m tsemlib_gb300.build`")
            _build.build(variant=VARIANT)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc, allow=()):
    if rc != 0 and rc not in allow:
        raise TsemError(rc, lib().tsem_last_error().decode())
    return rc


def ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)
    return ctypes.c_void_p(int(a))


def stream_ptr(stream):
    """A CUDA stream handle for the C ABI: None = the library's own stream; torch's
    legacy default stream (handle 0) is passed as cudaStreamLegacy."""
    if stream is None:
        return None
    h = int(stream)
    return ctypes.c_void_p(h if h != 0 else 1)


def c_array(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)
