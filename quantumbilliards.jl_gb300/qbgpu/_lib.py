"""ctypes binding of libqbgpu (the C ABI declared in include/qbgpu.h).

This is the Python counterpart of the Julia ``ccall`` shim: plain pointers and
sizes, no torch types. The product has no CPU fallback: if the shared library
is missing or cannot be loaded, importing this module raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("QBGPU_LIB", _HERE / "libqbgpu.so"))

QBG_OK, QBG_EINVAL, QBG_ENOMEM, QBG_EBUDGET, QBG_ESINGULAR, QBG_ETIMEOUT, QBG_ECUDA, QBG_ENOTSUP = range(8)
QBG_FORM_DLP, QBG_FORM_CFIE = 0, 1
QBG_PREC_FP64, QBG_PREC_MIXED, QBG_PREC_FP32 = 0, 1, 2
QBG_PTR_DEVICE = 1
QBG_V_PER_DISK = 2
QBG_SPLIT_LO = 4
QBG_EBIM_FULL = 8


def prec_code(p) -> int:
    """'fp64' | 'mixed' | 'fp32' (or False/True for fp64/mixed) -> QBG_PREC_*."""
    if p is None or p is False or p == "fp64":
        return QBG_PREC_FP64
    if p is True or p == "mixed":
        return QBG_PREC_MIXED
    if p == "fp32":
        return QBG_PREC_FP32
    if p in (0, 1, 2):
        return int(p)
    raise ValueError(f"unknown precision form {p!r}")

STATUS_NAMES = {0: "QBG_OK", 1: "QBG_EINVAL", 2: "QBG_ENOMEM", 3: "QBG_EBUDGET", 4: "QBG_ESINGULAR",
                5: "QBG_ETIMEOUT", 6: "QBG_ECUDA", 7: "QBG_ENOTSUP"}


class QBGError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"qbgpu: {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class GeomDesc(C.Structure):
    _fields_ = [("form", C.c_int32), ("ncomp", C.c_int32), ("comp_offsets", C.POINTER(C.c_int64)),
                ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)),
                ("dx", C.POINTER(C.c_double)), ("dy", C.POINTER(C.c_double)),
                ("ddx", C.POINTER(C.c_double)), ("ddy", C.POINTER(C.c_double)),
                ("ts", C.POINTER(C.c_double)), ("ws", C.POINTER(C.c_double)),
                ("m", C.c_int64), ("norb", C.c_int32), ("fund", C.POINTER(C.c_int64)),
                ("orbit", C.POINTER(C.c_int64)), ("orbit_scale", C.POINTER(C.c_double)),
                ("quad", C.c_int32), ("alpert_a", C.c_int32), ("alpert_j", C.c_int32),
                ("alpert_ninterp", C.c_int32), ("alpert_w", C.POINTER(C.c_double)),
                ("alpert_off", C.POINTER(C.c_int64)), ("alpert_wt", C.POINTER(C.c_double)),
                ("alpert_nodes", C.POINTER(C.c_double))]


class ChebParams(C.Structure):
    _fields_ = [("n_panels_h", C.c_int32), ("M_h", C.c_int32), ("n_panels_j", C.c_int32), ("M_j", C.c_int32)]


class BeynOpts(C.Structure):
    _fields_ = [("flags", C.c_int32), ("max_refine", C.c_int32), ("refine_tol", C.c_double), ("nb", C.c_int32),
                ("eval_mode", C.c_int32), ("cheb", ChebParams), ("fp32_sweeps", C.c_int32),
                ("solve_block", C.c_int32), ("node_chunk", C.c_int32), ("resid_engine", C.c_int32)]


class BeynStats(C.Structure):
    _fields_ = [("refine_sweeps", C.c_int32), ("refine_residual", C.c_double), ("singular", C.c_int32),
                ("ms_assemble", C.c_double), ("ms_factor", C.c_double), ("ms_solve", C.c_double),
                ("nhist", C.c_int32), ("refine_history", C.c_double * 8), ("ms_residual", C.c_double),
                ("n_residual", C.c_int32), ("nfp32", C.c_int32), ("fp32_history", C.c_double * 4),
                ("ms_solves", C.c_double), ("n_solves", C.c_int32)]


class ServeOpts(C.Structure):
    _fields_ = [("hbm_budget", C.c_int64), ("workers", C.c_int32), ("max_batch", C.c_int32),
                ("max_sweeps", C.c_int32)]


class RequestDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("geom", C.c_void_p), ("prec", C.c_int32),
                ("k0_re", C.c_double), ("k0_im", C.c_double), ("R", C.c_double), ("nq", C.c_int32),
                ("L", C.c_int64), ("V", C.c_void_p), ("A0", C.c_void_p), ("A1", C.c_void_p),
                ("k", C.c_double), ("out_A", C.c_void_p), ("out_dA", C.c_void_p), ("out_ddA", C.c_void_p),
                ("ks", C.c_void_p), ("nk", C.c_int64), ("sig", C.c_void_p)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("batched", C.c_int32), ("queue_ms", C.c_double), ("run_ms", C.c_double)]


# symbol -> (restype, argtypes); the list is the ABI surface the tests check
_SIGS = {
    "qbg_version": (C.c_int32, [C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "qbg_last_error": (C.c_size_t, [C.c_char_p, C.c_size_t]),
    "qbg_device_sync": (C.c_int32, []),
    "qbg_geom_create": (C.c_int32, [C.POINTER(GeomDesc), C.POINTER(C.c_void_p)]),
    "qbg_geom_destroy": (C.c_int32, [C.c_void_p]),
    "qbg_geom_dim": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int64)]),
    "qbg_assemble": (C.c_int32, [C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                 C.POINTER(C.c_void_p)]),
    "qbg_assemble_cheb": (C.c_int32, [C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.c_int32, C.c_int32,
                                      C.c_int32, C.POINTER(ChebParams), C.POINTER(C.c_void_p)]),
    "qbg_assemble_noalloc": (C.c_int32, [C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.c_int32, C.c_int32,
                                         C.POINTER(C.c_void_p)]),
    "qbg_beyn_create": (C.c_int32, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                    C.POINTER(BeynOpts), C.POINTER(C.c_void_p)]),
    "qbg_beyn_moments": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                     C.POINTER(BeynStats)]),
    "qbg_beyn_moments_qr": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int64, C.c_void_p,
                                        C.c_void_p, C.POINTER(BeynStats)]),
    "qbg_beyn_B": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p,
                               C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                               C.POINTER(BeynStats)]),
    "qbg_beyn_destroy": (C.c_int32, [C.c_void_p]),
    "qbg_set_tc_wait_limit": (C.c_int32, [C.c_int64]),
    "qbg_dense_inverse": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                      C.POINTER(C.c_double), C.c_void_p]),
    "qbg_set_lu_plan": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32]),
    "qbg_get_lu_plan": (C.c_int32, [C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "qbg_clear_tc_error": (C.c_int32, []),
    "qbg_sigma_min": (C.c_int32, [C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_double)]),
    "qbg_ebim_eig": (C.c_int32, [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int32,
                                 C.c_int32, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "qbg_newton_refine": (C.c_int32, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_double,
                                      C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "qbg_adjoint_fredholm": (C.c_int32, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_int32]),
    "qbg_solve_vect": (C.c_int32, [C.c_void_p, C.c_double, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]),
    "qbg_small_eig": (C.c_int32, [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "qbg_ebim_solve": (C.c_int32, [C.c_void_p, C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_int32,
                                   C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int32),
                                   C.POINTER(C.c_int32)]),
    "qbg_bessel01": (C.c_int32, [C.POINTER(C.c_double), C.c_int64, C.c_int32, C.POINTER(C.c_double)]),
    "qbg_cgemm_c64": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_float), C.c_void_p,
                                  C.c_int64, C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.c_void_p, C.c_int64,
                                  C.c_int32]),
    "qbg_set_gemm_engine": (C.c_int32, [C.c_int32]),
    "qbg_zgemm_sub_tc": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p,
                                     C.c_int64, C.c_void_p, C.c_int64, C.c_int32]),
    "qbg_residual_c64": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "qbg_serve_create": (C.c_int32, [C.POINTER(ServeOpts), C.POINTER(C.c_void_p)]),
    "qbg_serve_submit": (C.c_int32, [C.c_void_p, C.POINTER(RequestDesc), C.POINTER(C.c_int64)]),
    "qbg_serve_poll": (C.c_int32, [C.c_void_p, C.c_int64, C.POINTER(C.c_int32)]),
    "qbg_serve_wait": (C.c_int32, [C.c_void_p, C.c_int64, C.c_double, C.POINTER(RequestResult)]),
    "qbg_serve_destroy": (C.c_int32, [C.c_void_p]),
    "qbg_launch_count": (C.c_int32, [C.POINTER(C.c_uint64)]),
    "qbg_pool_release": (C.c_int32, []),
    "qbg_pool_stats": (C.c_int32, [C.POINTER(C.c_uint64)] * 4),
    "qbg_candidate_residuals": (C.c_int32, [C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.c_void_p,
                                            C.POINTER(ChebParams), C.POINTER(C.c_double)]),
    "qbg_cheb_autotune": (C.c_int32, [C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.c_double, C.c_int32,
                                      C.c_int32, C.c_int32, C.POINTER(ChebParams), C.POINTER(C.c_double)]),
    "qbg_beyn_create_disks": (C.c_int32, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int32,
                                          C.c_int32, C.c_int32, C.c_void_p, C.POINTER(C.c_void_p)]),
}

_lib = None
_shutting_down = False


def _mark_shutdown():
    global _shutting_down
    _shutting_down = True


import atexit as _atexit  # noqa: E402

# handles are released explicitly or by the garbage collector while the
# process is alive; after interpreter shutdown starts, the CUDA runtime may
# already be torn down, so destructors must not call into the library.
_atexit.register(_mark_shutdown)


def alive() -> bool:
    return _lib is not None and not _shutting_down


def load(path: Path | None = None):
    """Load (once) and return the shared library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"libqbgpu.so not found at {p}; build it with __graft_entry__.build()")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_SIGS)


def last_error() -> str:
    lib = load()
    buf = C.create_string_buffer(2048)
    lib.qbg_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int):
    if status != QBG_OK:
        raise QBGError(status, last_error())


def dptr(a: np.ndarray, ctype=C.c_double):
    return a.ctypes.data_as(C.POINTER(ctype))


def vptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)
