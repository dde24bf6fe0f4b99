"""ctypes binding of libemfa_cuda.so (include/emfa_cuda.h).

This is the reference-facing C ABI called from Python; tests and the bench
drive the GPU path only through these entry points.  Device buffers are
passed as raw pointers (torch tensors' data_ptr()).  Loading fails loudly if
the library was not built: there is no fallback path.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libemfa_cuda.so")
HEADER = os.path.join(HERE, "..", "include", "emfa_cuda.h")

EMFA_OK = 0
STATUS = {0: "EMFA_OK", 1: "EMFA_ERR_INVALID", 2: "EMFA_ERR_CUDA", 3: "EMFA_ERR_OOM",
          4: "EMFA_ERR_NOT_CONVERGED", 5: "EMFA_ERR_MESH", 6: "EMFA_ERR_UNSUPPORTED", 7: "EMFA_ERR_TIMEOUT"}
EMFA_F32, EMFA_F64 = 0, 1
EMFA_EFIE, EMFA_CFIE = 0, 1
EMFA_GMRES, EMFA_BICGSTAB, EMFA_LU = 0, 1, 2
EMFA_MV_AUTO, EMFA_MV_F64, EMFA_MV_F32, EMFA_MV_TF32, EMFA_MV_F16X = 0, 1, 2, 3, 4


class FillParams(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("precision", ctypes.c_int), ("freq", ctypes.c_double),
                ("alpha", ctypes.c_double), ("sigma_re", ctypes.c_double), ("sigma_im", ctypes.c_double),
                ("edm_mode", ctypes.c_int), ("discretisation", ctypes.c_int)]


class SolverParams(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("restart", ctypes.c_int), ("max_iter", ctypes.c_int),
                ("tol", ctypes.c_double), ("tol_absolute", ctypes.c_int), ("matvec", ctypes.c_int),
                ("max_refine", ctypes.c_int), ("orth", ctypes.c_int), ("inner_reduction", ctypes.c_double),
                ("basis", ctypes.c_int)]


class MlfmaParams(ctypes.Structure):
    _fields_ = [("freq", ctypes.c_double), ("alpha", ctypes.c_double), ("box_threshold", ctypes.c_double),
                ("precond", ctypes.c_int), ("row_threshold", ctypes.c_double), ("col_threshold", ctypes.c_double),
                ("truncation", ctypes.c_int)]


class Request(ctypes.Structure):
    _fields_ = [("verts", ctypes.c_void_p), ("n_vert", ctypes.c_int), ("tris", ctypes.c_void_p), ("n_tri", ctypes.c_int),
                ("kind", ctypes.c_int), ("method", ctypes.c_int), ("freq", ctypes.c_double), ("alpha", ctypes.c_double),
                ("angles", ctypes.c_void_p), ("n_inc", ctypes.c_int), ("rcs_dirs", ctypes.c_void_p),
                ("n_dir", ctypes.c_int), ("per_rhs_dirs", ctypes.c_int), ("tol", ctypes.c_double),
                ("max_iter", ctypes.c_int), ("box_threshold", ctypes.c_double), ("arrival_s", ctypes.c_double),
                ("rcs_out", ctypes.c_void_p)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("method", ctypes.c_int), ("n_rwg", ctypes.c_int),
                ("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("max_rel_residual", ctypes.c_double),
                ("t_arrive", ctypes.c_double), ("t_start", ctypes.c_double), ("t_done", ctypes.c_double),
                ("hbm_estimate", ctypes.c_size_t), ("lane", ctypes.c_int)]


class ServeOpts(ctypes.Structure):
    _fields_ = [("lanes", ctypes.c_int), ("hbm_budget", ctypes.c_size_t), ("dense_max", ctypes.c_int),
                ("realtime", ctypes.c_int), ("max_wait_s", ctypes.c_double)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("cycles", ctypes.c_int), ("converged", ctypes.c_int),
                ("max_rel_residual", ctypes.c_double), ("seconds", ctypes.c_double)]


class EmfaError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


_lib = None
vp = ctypes.c_void_p
ci = ctypes.c_int
sz = ctypes.c_size_t
dp = ctypes.POINTER(ctypes.c_double)
ip = ctypes.POINTER(ctypes.c_int)

_SIGS = {
    "emfa_status_string": (ctypes.c_char_p, [ci]),
    "emfa_last_error": (ctypes.c_char_p, [vp]),
    "emfa_version": (ctypes.c_char_p, []),
    "emfa_ctx_create": (ci, [ci, sz, ctypes.POINTER(vp)]),
    "emfa_ctx_destroy": (ci, [vp]),
    "emfa_ctx_memory": (ci, [vp, ctypes.POINTER(sz), ctypes.POINTER(sz), ctypes.POINTER(sz)]),
    "emfa_ctx_launch_count": (ci, [vp, ctypes.POINTER(ctypes.c_int64)]),
    "emfa_autotune_query": (ci, [ci, ci, ci, ip, ctypes.POINTER(ctypes.c_float)]),
    "emfa_autotune_clear": (ci, []),
    "emfa_ctx_synchronize": (ci, [vp]),
    "emfa_ctx_stream": (ci, [vp, ctypes.POINTER(vp)]),
    "emfa_device_alloc": (ci, [vp, sz, ctypes.POINTER(vp)]),
    "emfa_device_free": (ci, [vp, vp]),
    "emfa_memcpy": (ci, [vp, vp, vp, sz, ci]),
    "emfa_build_rwg": (ci, [vp, ci, vp, ci, ip]),
    "emfa_geom_create": (ci, [vp, vp, ci, vp, ci, vp, ci, ctypes.POINTER(vp)]),
    "emfa_geom_destroy": (ci, [vp]),
    "emfa_geom_size": (ci, [vp, ip, ip, ip]),
    "emfa_fill_z": (ci, [vp, vp, ctypes.POINTER(FillParams), vp, sz, vp]),
    "emfa_fill_v": (ci, [vp, vp, ctypes.POINTER(FillParams), vp, ci, vp, vp]),
    "emfa_matvec": (ci, [vp, ci, ci, vp, ci, vp, ci, vp, vp]),
    "emfa_matvec_tf32_noalloc": (ci, [vp, ci, vp, ci, vp, vp]),
    "emfa_ctx_set_kernel_timing": (ci, [vp, ci]),
    "emfa_serve": (ci, [ci, ctypes.POINTER(Request), ci, ctypes.POINTER(ServeOpts), ctypes.POINTER(RequestResult)]),
    "emfa_serve_simulate": (ci, [vp, vp, vp, ci, ctypes.POINTER(ServeOpts), vp, vp]),
    "emfa_diag_sincospi": (ci, [vp, ci, vp, vp, vp]),
    "emfa_diag_wait_timeout": (ci, [vp, ctypes.POINTER(ci)]),
    "emfa_dump_save": (ci, [ctypes.c_char_p, ctypes.c_char_p, ci, sz, sz, ctypes.c_double, vp, ci]),
    "emfa_dump_info": (ci, [ctypes.c_char_p, ctypes.c_char_p, ip, ctypes.POINTER(sz), ctypes.POINTER(sz),
                            ctypes.POINTER(ctypes.c_double)]),
    "emfa_dump_load": (ci, [ctypes.c_char_p, vp, sz, ci]),
    "emfa_residual": (ci, [vp, ci, ci, vp, ci, vp, vp, ci, vp, vp]),
    "emfa_ctx_kernel_time": (ci, [vp, ci, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_double)]),
    "emfa_solve": (ci, [vp, ci, vp, ci, vp, ci, vp, ctypes.POINTER(SolverParams), ctypes.POINTER(SolveInfo), vp]),
    "emfa_rcs": (ci, [vp, vp, ctypes.POINTER(FillParams), vp, ci, vp, ci, ci, vp, vp]),
    "emfa_mlfma_plan": (ci, [vp, ci, vp, ci, ctypes.POINTER(MlfmaParams), ip, vp, ci, vp, vp]),
    "emfa_mlfma_create": (ci, [vp, vp, ctypes.POINTER(MlfmaParams), ctypes.POINTER(vp)]),
    "emfa_mlfma_destroy": (ci, [vp]),
    "emfa_mlfma_precond_csr": (ci, [vp, ctypes.POINTER(sz), vp, vp, vp]),
    "emfa_mlfma_precond_lists": (ci, [vp, ip, ctypes.POINTER(sz), ctypes.POINTER(sz), vp, vp, vp, vp, vp]),
    "emfa_mlfma_info": (ci, [vp, ip, vp, vp, ctypes.POINTER(sz), vp]),
    "emfa_mlfma_apply": (ci, [vp, vp, vp, ci, vp]),
    "emfa_mlfma_apply_part": (ci, [vp, vp, vp, ci, vp]),
    "emfa_mlfma_fill_v": (ci, [vp, vp, ci, vp, vp]),
    "emfa_mlfma_solve": (ci, [vp, vp, ci, vp, ctypes.POINTER(SolverParams), ctypes.POINTER(SolveInfo), vp]),
    "emfa_mlfma_unpermute": (ci, [vp, vp, ci, vp, vp]),
    "emfa_dense_rcs": (ci, [vp, vp, ci, vp, ci, ctypes.POINTER(FillParams), vp, ci, ctypes.POINTER(SolverParams),
                            vp, ci, ci, vp, vp, ctypes.POINTER(SolveInfo)]),
}


def header_symbols() -> list[str]:
    """Every function the public header declares."""
    txt = open(HEADER).read()
    return sorted(set(n for n in re.findall(r"\b(emfa_[a-z0-9_]+)\s*\(", txt) if not n.endswith("_t")))


def lib():
    """Load the in-tree library (built by emfa_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libemfa_cuda.so is not built (run emfa_gb300.build.build()): %s" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status, ctx=None):
    if status != EMFA_OK:
        msg = lib().emfa_last_error(ctx)
        raise EmfaError(status, (msg or b"").decode(errors="replace"))
    return status
