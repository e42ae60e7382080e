"""ctypes binding of libcmsl_gb.so (include/cmsl.h).

The library is built in-tree by ``cmsl_gb300.build.build()``.  There is no
fallback: if the shared object is missing or fails to load, every entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcmsl_gb.so")

CMSL_OK = 0
STATUS_NAMES = {0: "CMSL_OK", 1: "CMSL_ERR_ARG", 2: "CMSL_ERR_CUDA", 3: "CMSL_ERR_IO", 4: "CMSL_ERR_PCG",
                5: "CMSL_ERR_STATE", 6: "CMSL_ERR_NOMEM"}
FP64, FP32_REFINED = 0, 1
DIRICHLET, NEUMANN = 0, 1
CRIT_REF, CRIT_RELRES = 0, 1
INNER_AUTO, INNER_PCG, INNER_DIRECT = 0, 1, 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class Material(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("alpha", "beta", "gamma", "g", "a0", "kappa", "L", "eps_r")]


class FilmDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("del_h", C.c_double), ("del_t", C.c_double),
        ("dep_flag", C.c_int), ("zbc", C.c_int), ("eps_0_nd", C.c_double),
        ("n_grains", C.c_int),
        ("omega", _ip), ("grain_mat", _ip), ("TR", _dp), ("is_interface", _ip),
        ("mats", Material * 3),
        ("precision", C.c_int), ("pcg_crit", C.c_int),
        ("tol_abs", C.c_double), ("tol_rel", C.c_double), ("max_iter", C.c_int),
        ("refine_tol", C.c_double), ("max_refine", C.c_int),
        ("inner_tol", C.c_double), ("inner_max_iter", C.c_int), ("warm_start", C.c_int),
        ("inner_solver", C.c_int),
    ]


class CmslError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run cmsl_gb300.build.build() (nvcc, sm_103a) first")
    L = C.CDLL(LIB_PATH)
    L.cmsl_last_error.restype = C.c_char_p
    L.cmsl_version.restype = C.c_char_p
    fp = C.c_void_p
    L.cmsl_film_create.argtypes = [C.POINTER(FilmDesc), C.POINTER(fp)]
    L.cmsl_film_destroy.argtypes = [fp]
    L.cmsl_film_set_state.argtypes = [fp, C.POINTER(_dp), _dp]
    L.cmsl_film_get_state.argtypes = [fp, C.POINTER(_dp), _dp]
    L.cmsl_film_run.argtypes = [fp, C.c_int, _dp, _ip, C.c_void_p]
    L.cmsl_film_sync.argtypes = [fp]
    L.cmsl_film_get_rows.argtypes = [fp, C.c_int, C.c_int, _dp]
    L.cmsl_film_get_iters.argtypes = [fp, C.c_int, _ip, _ip]
    L.cmsl_film_tdgl_step.argtypes = [fp, C.c_double]
    L.cmsl_film_depol.argtypes = [fp, _ip, _ip]
    L.cmsl_film_apply_operator.argtypes = [fp, _dp, _dp]
    L.cmsl_film_efield.argtypes = [fp, _dp, _dp, _dp]
    L.cmsl_film_diag_inv.argtypes = [fp, _dp]
    L.cmsl_film_time_kernels.argtypes = [fp, C.c_int, C.c_void_p, _dp]
    L.cmsl_film_device_bytes.argtypes = [fp, C.POINTER(C.c_size_t)]
    L.cmsl_film_inner_solver.argtypes = [fp, C.POINTER(C.c_int)]
    L.cmsl_film_autotune.argtypes = [fp, C.POINTER(C.c_int32)]
    L.cmsl_film_tile_config.argtypes = [fp, C.POINTER(C.c_int32)]
    L.cmsl_film_checkpoint_write.argtypes = [fp, C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_double]
    L.cmsl_film_checkpoint_read.argtypes = [fp, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), _dp, _dp]
    L.cmsl_film_loop_gradient.argtypes = [fp, C.c_int, _dp, _ip, _dp, C.c_int, C.c_int, _dp, _dp]
    L.cmsl_batch_create.argtypes = [C.POINTER(FilmDesc), C.c_int, C.POINTER(fp)]
    L.cmsl_batch_destroy.argtypes = [fp]
    L.cmsl_batch_set_state.argtypes = [fp, C.c_int, C.POINTER(_dp), _dp]
    L.cmsl_batch_get_state.argtypes = [fp, C.c_int, C.POINTER(_dp), _dp]
    L.cmsl_batch_run.argtypes = [fp, C.c_int, _dp, _ip, C.c_void_p]
    L.cmsl_batch_sync.argtypes = [fp, _ip]
    L.cmsl_batch_get_rows.argtypes = [fp, C.c_int, C.c_int, C.c_int, _dp]
    L.cmsl_batch_get_iters.argtypes = [fp, C.c_int, C.c_int, _ip, _ip]
    L.cmsl_batch_time_kernels.argtypes = [fp, C.c_int, C.c_void_p, _dp]
    L.cmsl_batch_device_bytes.argtypes = [fp, C.POINTER(C.c_size_t)]
    L.cmsl_batch_inner_solver.argtypes = [fp, C.POINTER(C.c_int)]
    L.cmsl_batch_autotune.argtypes = [fp, C.POINTER(C.c_int32)]
    L.cmsl_batch_tile_config.argtypes = [fp, C.POINTER(C.c_int32)]
    L.cmsl_host_alloc.argtypes = [C.c_size_t, C.POINTER(C.c_void_p)]
    L.cmsl_host_free.argtypes = [C.c_void_p]
    L.cmsl_film_depol_device.argtypes = [fp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, _ip, _ip]
    L.cmsl_depol_solve_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double,
                                           C.c_void_p, _dp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_double, C.c_double, C.c_int, C.c_int, C.c_void_p, _ip, _ip]
    _lib = L
    return L


def check(status: int) -> None:
    if status != CMSL_OK:
        raise CmslError(status, lib().cmsl_last_error().decode(errors="replace"))


# Every function include/cmsl.h declares; the CPU test checks the export list.
EXPORTS = [
    "cmsl_last_error", "cmsl_version", "cmsl_film_create", "cmsl_film_destroy", "cmsl_film_set_state",
    "cmsl_film_get_state", "cmsl_host_alloc", "cmsl_host_free", "cmsl_film_run", "cmsl_film_sync",
    "cmsl_film_get_rows", "cmsl_film_get_iters",
    "cmsl_film_tdgl_step", "cmsl_film_depol", "cmsl_film_depol_device", "cmsl_film_apply_operator",
    "cmsl_film_efield",
    "cmsl_film_diag_inv", "cmsl_film_time_kernels", "cmsl_film_device_bytes", "cmsl_film_inner_solver", "cmsl_film_autotune",
    "cmsl_film_tile_config",
    "cmsl_film_checkpoint_write",
    "cmsl_film_checkpoint_read", "cmsl_film_loop_gradient",
    "cmsl_batch_create",
    "cmsl_batch_destroy", "cmsl_batch_set_state", "cmsl_batch_get_state", "cmsl_batch_run", "cmsl_batch_sync",
    "cmsl_batch_get_rows", "cmsl_batch_get_iters", "cmsl_batch_time_kernels", "cmsl_batch_device_bytes",
    "cmsl_batch_inner_solver", "cmsl_batch_autotune", "cmsl_batch_tile_config",
    "cmsl_depol_solve_noalloc",
]
