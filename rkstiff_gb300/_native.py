"""ctypes binding of librkstiff_gb300 (the C ABI declared in include/rkstiff_gb300.h).

The library is required: importing the solver path without it raises, there is no
CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import _build

# enums (include/rkstiff_gb300.h)
RK_IF34, RK_ETD35, RK_ETD34, RK_IF45DP, RK_ETD4, RK_ETD5, RK_IF4 = range(7)
METHOD_IDS = {"IF34": RK_IF34, "ETD35": RK_ETD35, "ETD34": RK_ETD34, "IF45DP": RK_IF45DP,
              "ETD4": RK_ETD4, "ETD5": RK_ETD5, "IF4": RK_IF4}
RK_FP64, RK_FP32 = 0, 1
RK_NL_NONE, RK_NL_UUX, RK_NL_NLS, RK_NL_ALLEN_CAHN = 0, 1, 2, 3
RK_RUN_EVOLVE, RK_RUN_STEP = 0, 1
RK_ST_RUNNING, RK_ST_DONE, RK_ST_MAX_LOOPS, RK_ST_MIN_STEP = -1, 0, 1, 2
RK_ST_ITER_CAP, RK_ST_SNAP_FULL, RK_ST_STEP_DONE, RK_ST_BAD_SIZE, RK_ST_WAIT_TIMEOUT = 4, 5, 6, 7, 8
RK_OK, RK_E_ARG, RK_E_CUDA, RK_E_UNSUPPORTED, RK_E_SIZE = 0, -1, -2, -3, -4
RK_TW_N = 8192
ABI_VERSION = 2
RK_PLACE_AUTO, RK_PLACE_GLOBAL, RK_PLACE_SMEM_STATE, RK_PLACE_SMEM_ALL, RK_PLACE_SMEM_U = -1, 0, 1, 2, 3

# number of stage arrays and coefficient arrays per method (mirrors rk_evolve.cuh Traits)
STAGE_ARRAYS = {RK_ETD35: 6, RK_ETD5: 6, RK_ETD34: 5, RK_ETD4: 4, RK_IF34: 5, RK_IF4: 4, RK_IF45DP: 7}


class RkController(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("epsilon", "incr_f", "decr_f", "safety_f", "adapt_cutoff", "minh")]


class RkEtdConfig(ctypes.Structure):
    _fields_ = [("modecutoff", ctypes.c_double), ("contour_radius", ctypes.c_double),
                ("contour_points", ctypes.c_int32), ("contour_at_zero", ctypes.c_int32)]


class RkBatch(ctypes.Structure):
    _fields_ = [
        ("method", ctypes.c_int32), ("precision", ctypes.c_int32), ("coef_complex", ctypes.c_int32),
        ("nl_kind", ctypes.c_int32), ("nl_coef", ctypes.c_double), ("n_inst", ctypes.c_int64),
        ("n_max", ctypes.c_int32), ("reserved0", ctypes.c_int32),
        ("n", ctypes.c_void_p), ("mode_off", ctypes.c_void_p), ("order", ctypes.c_void_p),
        ("lin_op", ctypes.c_void_p), ("kx", ctypes.c_void_p), ("u", ctypes.c_void_p), ("state", ctypes.c_void_p),
        ("slab", ctypes.c_void_p), ("slab_off", ctypes.c_void_p), ("twiddle", ctypes.c_void_p),
        ("queue", ctypes.c_void_p), ("store_freq", ctypes.c_int32), ("snap_cap", ctypes.c_int32),
        ("snap_u", ctypes.c_void_p), ("snap_t", ctypes.c_void_p), ("max_steps", ctypes.c_int64),
        ("run_mode", ctypes.c_int32), ("threads", ctypes.c_int32),
        ("ctl", RkController), ("etd", RkEtdConfig),
        ("n_classes", ctypes.c_int32), ("placement", ctypes.c_int32),
        ("class_n", ctypes.c_void_p), ("class_start", ctypes.c_void_p),
        ("class_threads", ctypes.c_void_p), ("class_place", ctypes.c_void_p),
        ("class_groups", ctypes.c_void_p),
        ("attempt_log", ctypes.c_void_p), ("log_cap", ctypes.c_int32), ("mlp_target", ctypes.c_float),
        ("mlp", ctypes.c_void_p),
        ("ring_data", ctypes.c_void_p), ("ring_slot_bytes", ctypes.c_int64), ("ring_slots", ctypes.c_int32),
        ("ring_timeout_ms", ctypes.c_int32), ("ring_head", ctypes.c_void_p), ("ring_tail", ctypes.c_void_p),
        ("coef_blocks", ctypes.c_int32), ("ladder", ctypes.c_int32),
    ]


RK_RING_HEADER = 32


class RkRing(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("head", ctypes.c_void_p), ("tail", ctypes.c_void_p),
                ("slot_bytes", ctypes.c_int64), ("slots", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class RkTerm(ctypes.Structure):
    _fields_ = [("coef", ctypes.c_void_p), ("v", ctypes.c_void_p), ("w", ctypes.c_double)]


class RkDenseBatch(ctypes.Structure):
    _fields_ = [
        ("method", ctypes.c_int32), ("n", ctypes.c_int32), ("n_inst", ctypes.c_int64),
        ("nl_kind", ctypes.c_int32), ("err_eigen", ctypes.c_int32),
        ("eig", ctypes.c_void_p), ("S", ctypes.c_void_p), ("Sinv", ctypes.c_void_p), ("shift", ctypes.c_void_p),
        ("u", ctypes.c_void_p), ("work", ctypes.c_void_p), ("state", ctypes.c_void_p),
        ("ctl", RkController), ("etd", RkEtdConfig), ("max_attempts", ctypes.c_int64),
    ]


class RkDenseEigBatch(ctypes.Structure):
    _fields_ = [
        ("method", ctypes.c_int32), ("n", ctypes.c_int32), ("n_inst", ctypes.c_int64),
        ("nl_kind", ctypes.c_int32), ("err_eigen", ctypes.c_int32),
        ("eig", ctypes.c_void_p), ("S", ctypes.c_void_p), ("Sinv", ctypes.c_void_p), ("shift", ctypes.c_void_p),
        ("u", ctypes.c_void_p), ("work", ctypes.c_void_p), ("state", ctypes.c_void_p),
        ("ctl", RkController), ("etd", RkEtdConfig), ("first", ctypes.c_int32), ("max_attempts", ctypes.c_int32),
    ]


RK_DENSE_NMAX, RK_DENSE_TILE = 128, 64
# rk_dense_state (128 bytes)
DENSE_STATE_DTYPE = np.dtype([
    ("t", "f8"), ("tf", "f8"), ("h", "f8"), ("h_coeff", "f8"), ("h_suggest", "f8"), ("s_last", "f8"),
    ("status", "i4"), ("cur", "i4"), ("numloops", "i4"), ("accept", "i4"), ("need_matrix", "i4"), ("error", "i4"),
    ("n1_fresh", "i4"), ("reserved_i", "i4"),
    ("steps", "i8"), ("attempts", "i8"), ("rejects", "i8"), ("nl_evals", "i8"), ("coeff_updates", "i8"),
    ("reserved", "i8"),
])
assert DENSE_STATE_DTYPE.itemsize == 128

# rk_inst_state as a NumPy record (128 bytes)
STATE_DTYPE = np.dtype([
    ("t", "f8"), ("tf", "f8"), ("h", "f8"), ("h_coeff", "f8"), ("h_used", "f8"), ("h_suggest", "f8"),
    ("s_last", "f8"), ("reserved_d", "f8"), ("status", "i4"), ("accept", "i4"), ("snap_count", "i4"),
    ("reserved_i", "i4"), ("steps", "i8"), ("attempts", "i8"), ("rejects", "i8"), ("nl_evals", "i8"),
    ("coeff_updates", "i8"), ("reserved_l", "i8"),
])
assert STATE_DTYPE.itemsize == 128

# every symbol the header declares
EXPORTS = ("rk_abi_version", "rk_last_error", "rk_fill_twiddles", "rk_slab_bytes", "rk_slab_bytes_blocks",
           "rk_num_coeffs", "rk_coeffs",
           "rk_evolve", "rk_probe_fp32", "rk_evolve_noalloc", "rk_mlp_forward", "rk_mlp_grad", "rk_mlp_adam",
           "rk_mlp_pack", "rk_dense_work_bytes", "rk_dense_evolve", "rk_tf32x3_work_bytes", "rk_tf32x3_gemm",
           "rk_combine", "rk_error_s", "rk_cgemv", "rk_dense_eig_work_bytes", "rk_dense_eig_evolve",
           "rk_fourier_grid", "rk_cheb_grid", "rk_dx_fourier", "rk_dx_cheb_work_bytes", "rk_dx_cheb",
           "rk_ring_create", "rk_ring_take", "rk_ring_reset", "rk_ring_destroy", "rk_nls_lines", "rk_dht")
RK_LOG_FIELDS = 8
RK_MLP_IN, RK_MLP_H = 8, 64
RK_MLP_NPARAM = RK_MLP_H * RK_MLP_IN + RK_MLP_H + RK_MLP_H * RK_MLP_H + RK_MLP_H + RK_MLP_H + 1
RK_MLP_PACK_BYTES = (2 * RK_MLP_IN + 2 * RK_MLP_H + 4) * 4 + (RK_MLP_H * RK_MLP_IN + RK_MLP_H * RK_MLP_H + RK_MLP_H) * 2

_lib = None
_lock = threading.Lock()


class NativeError(RuntimeError):
    """A C entry point returned an error code."""


def load(build: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the shared library and declare its signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.build() if build else _build.lib_path()
        if not os.path.exists(path):
            raise RuntimeError(f"rkstiff_gb300 native library missing at {path}; run rkstiff_gb300._build.build()")
        lib = ctypes.CDLL(path)
        vp, i32, i64, dbl = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
        lib.rk_abi_version.restype = ctypes.c_int
        lib.rk_last_error.restype = ctypes.c_char_p
        lib.rk_fill_twiddles.argtypes = [vp, vp, vp]
        lib.rk_fill_twiddles.restype = ctypes.c_int
        lib.rk_slab_bytes.argtypes = [i32, i32, i32, i64]
        lib.rk_slab_bytes.restype = i64
        lib.rk_slab_bytes_blocks.argtypes = [i32, i32, i32, i64, i32]
        lib.rk_slab_bytes_blocks.restype = i64
        lib.rk_num_coeffs.argtypes = [i32]
        lib.rk_num_coeffs.restype = ctypes.c_int
        lib.rk_coeffs.argtypes = [i32, i32, i32, i64, vp, dbl, ctypes.POINTER(RkEtdConfig), vp, vp]
        lib.rk_coeffs.restype = ctypes.c_int
        lib.rk_evolve.argtypes = [ctypes.POINTER(RkBatch), vp]
        lib.rk_evolve.restype = ctypes.c_int
        lib.rk_probe_fp32.argtypes = [vp, i32, i32, i32, vp]
        lib.rk_probe_fp32.restype = ctypes.c_int
        lib.rk_evolve_noalloc.argtypes = [ctypes.POINTER(RkBatch), vp]
        lib.rk_evolve_noalloc.restype = ctypes.c_int
        f32 = ctypes.c_float
        lib.rk_mlp_forward.argtypes = [vp, vp, i64, vp, vp]
        lib.rk_mlp_grad.argtypes = [vp, vp, vp, i64, f32, vp, vp, vp]
        lib.rk_mlp_adam.argtypes = [vp, vp, vp, vp, i64, f32, f32, f32, f32, vp]
        lib.rk_mlp_pack.argtypes = [vp, vp, vp, vp, vp]
        for fn in (lib.rk_mlp_forward, lib.rk_mlp_grad, lib.rk_mlp_adam, lib.rk_mlp_pack):
            fn.restype = ctypes.c_int
        lib.rk_dense_work_bytes.argtypes = [i64]
        lib.rk_dense_work_bytes.restype = i64
        lib.rk_dense_eig_work_bytes.argtypes = [i64]
        lib.rk_dense_eig_work_bytes.restype = i64
        lib.rk_dense_eig_evolve.argtypes = [ctypes.POINTER(RkDenseEigBatch), vp]
        lib.rk_dense_eig_evolve.restype = ctypes.c_int
        lib.rk_dense_evolve.argtypes = [ctypes.POINTER(RkDenseBatch), vp]
        lib.rk_dense_evolve.restype = ctypes.c_int
        lib.rk_tf32x3_work_bytes.argtypes = [i64, i64]
        lib.rk_tf32x3_work_bytes.restype = i64
        lib.rk_tf32x3_gemm.argtypes = [vp, vp, vp, i64, i64, vp, vp]
        lib.rk_tf32x3_gemm.restype = ctypes.c_int
        lib.rk_combine.argtypes = [i32, i32, i64, ctypes.POINTER(RkTerm), i32, vp, vp]
        lib.rk_combine.restype = ctypes.c_int
        lib.rk_error_s.argtypes = [i32, i64, vp, vp, ctypes.POINTER(RkController), i32, vp, vp]
        lib.rk_error_s.restype = ctypes.c_int
        lib.rk_cgemv.argtypes = [i32, i64, vp, vp, vp, vp]
        lib.rk_cgemv.restype = ctypes.c_int
        lib.rk_fourier_grid.argtypes = [i32, i64, dbl, dbl, vp, vp, vp]
        lib.rk_cheb_grid.argtypes = [i64, dbl, dbl, vp, vp, vp]
        lib.rk_dx_fourier.argtypes = [i32, i32, i64, i64, vp, vp, vp, vp, vp]
        lib.rk_dx_cheb_work_bytes.argtypes = [i64]
        lib.rk_dx_cheb_work_bytes.restype = i64
        lib.rk_dx_cheb.argtypes = [i32, i64, i64, vp, vp, vp, vp, vp]
        for fn in (lib.rk_fourier_grid, lib.rk_cheb_grid, lib.rk_dx_fourier, lib.rk_dx_cheb):
            fn.restype = ctypes.c_int
        lib.rk_ring_create.argtypes = [i64, i64, ctypes.POINTER(RkRing)]
        lib.rk_ring_take.argtypes = [ctypes.POINTER(RkRing), i64, vp, i64]
        lib.rk_ring_reset.argtypes = [ctypes.POINTER(RkRing)]
        lib.rk_ring_destroy.argtypes = [ctypes.POINTER(RkRing)]
        for fn in (lib.rk_ring_create, lib.rk_ring_take, lib.rk_ring_reset, lib.rk_ring_destroy):
            fn.restype = ctypes.c_int
        lib.rk_nls_lines.argtypes = [i32, i32, i64, i64, i64, i64, dbl, vp, vp, vp, vp]
        lib.rk_nls_lines.restype = ctypes.c_int
        lib.rk_dht.argtypes = [i32, i32, i64, i64, vp, dbl, vp, vp, vp]
        lib.rk_dht.restype = ctypes.c_int
        if lib.rk_abi_version() != ABI_VERSION:
            raise RuntimeError("rkstiff_gb300 native library ABI mismatch")
        _lib = lib
        return lib


def check(rc: int, what: str) -> None:
    if rc != 0:
        msg = _lib.rk_last_error().decode() if _lib is not None else ""
        raise NativeError(f"{what} failed ({rc}): {msg}")
