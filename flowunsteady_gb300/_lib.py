"""ctypes binding of libvpmgpu.so (the C ABI declared in include/vpm_gpu.h).

The shared library is the product; this module only loads it.  If the
library is missing it is built from csrc/ with nvcc; if that is impossible
the import of the compute API fails loudly (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvpmgpu.so")

# Status codes
OK = 0
ERR_INVALID = -1
ERR_CAPACITY = -2
ERR_CUDA = -3
ERR_NONFINITE = -4
ERR_NOMEM = -5
ERR_UNSUPPORTED = -6
ERR_STATE = -7
ERR_INJECTED = -8

KERNEL_WINCKELMANS = 0
KERNEL_GAUSSIANERF = 1
PREC_FP64 = 0
PREC_FP32 = 1
PREC_FP32C = 2
INTEGRATION_EULER = 0
INTEGRATION_RK3 = 1
SFS_NONE = 0
SFS_DYNAMIC = 1
SFS_CONSTANT = 2
SFS_CLIP_BACKSCATTER = 1
SFS_FORCE_POSITIVE = 2
SFS_ANALYTIC_DSIGMA = 4
UJ_DIRECT = 0
UJ_TREE = 1
ORDER_AUTO = 0      # vpm_set_particle_order: Morton order for large fields and batches
ORDER_CALLER = 1    # the caller's order
RELAX_NONE = 0
RELAX_PEDRIZZETTI = 1

DIAG_NAMES = ["enstrophy", "impulse_x", "impulse_y", "impulse_z", "gamma_x", "gamma_y",
              "gamma_z", "cd_mean", "cd_std", "cd_zero_ratio", "cd_min", "cd_max",
              "sigma_mean", "nonfinite", "cd_skew", "cd_kurt"]
DIAG_COUNT = len(DIAG_NAMES)

# Every symbol include/vpm_gpu.h declares.
EXPORTS = [
    "vpm_scheme_default", "vpm_ctx_create", "vpm_ctx_destroy", "vpm_last_error",
    "vpm_ctx_set_stream", "vpm_get_time", "vpm_set_time", "vpm_set_particles", "vpm_append",
    "vpm_truncate", "vpm_get_np", "vpm_get_state", "vpm_get_sfs", "vpm_set_attributes",
    "vpm_get_attributes", "vpm_eval_UJ",
    "vpm_eval_UJ_targets", "vpm_get_UJ", "vpm_eval_sfs", "vpm_step", "vpm_diagnostics",
    "vpm_centroids", "vpm_ffv_direct", "vpm_fmm_default", "vpm_eval_UJ_fmm", "vpm_fmm_stats",
    "vpm_save", "vpm_load",
    "vpm_uj_device_async", "vpm_uj_device_noalloc", "vpm_batch_create", "vpm_batch_destroy",
    "vpm_batch_last_error", "vpm_batch_set_stream", "vpm_batch_set_field",
    "vpm_batch_get_field", "vpm_batch_eval_UJ", "vpm_batch_get_UJ", "vpm_batch_step",
    "vpm_batch_autotune", "vpm_batch_get_shapes",
    "vpm_autotune", "vpm_set_tile", "vpm_set_particle_order", "vpm_batch_set_particle_order",
    "vpm_measure_fma_peaks", "vpm_debug_fail_after", "vpm_debug_last_plan",
    "vpm_get_launch_count", "vpm_build_info",
]


class Fmm(ctypes.Structure):
    """Mirror of struct vpm_fmm (treecode settings)."""
    _fields_ = [("p", ctypes.c_int32), ("ncrit", ctypes.c_int32), ("theta", ctypes.c_double),
                ("sigma_factor", ctypes.c_double), ("local_order", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class Scheme(ctypes.Structure):
    """Mirror of struct vpm_scheme."""
    _fields_ = [
        ("kernel", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("integration", ctypes.c_int32),
        ("transposed", ctypes.c_int32),
        ("f", ctypes.c_double),
        ("g", ctypes.c_double),
        ("uinf", ctypes.c_double * 3),
        ("nu", ctypes.c_double),
        ("sfs", ctypes.c_int32),
        ("sfs_flags", ctypes.c_uint32),
        ("sfs_alpha", ctypes.c_double),
        ("sfs_rlxf", ctypes.c_double),
        ("sfs_minC", ctypes.c_double),
        ("sfs_maxC", ctypes.c_double),
        ("sfs_Cd", ctypes.c_double),
        ("relaxation", ctypes.c_int32),
        ("relax_nsteps", ctypes.c_int32),
        ("relax_factor", ctypes.c_double),
        ("uj_method", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("fmm", Fmm),
    ]


class Tile(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int32), ("tpt", ctypes.c_int32), ("chunk", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


FMM_STATS = ["cells", "leaves", "groups", "far_entries", "near_entries", "near_pairs",
             "far_evaluations", "local_terms"]


def default_fmm():
    f = Fmm()
    lib().vpm_fmm_default(ctypes.byref(f))
    return f


class VPMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_i64 = ctypes.c_int64
_vp = ctypes.c_void_p


def _declare(lib):
    P = ctypes.POINTER
    sig = {
        "vpm_scheme_default": (None, [P(Scheme)]),
        "vpm_ctx_create": (ctypes.c_int, [ctypes.c_int, _i64, P(_vp)]),
        "vpm_ctx_destroy": (ctypes.c_int, [_vp]),
        "vpm_last_error": (ctypes.c_int, [_vp, ctypes.c_char_p, _i64]),
        "vpm_ctx_set_stream": (ctypes.c_int, [_vp, _vp]),
        "vpm_get_time": (ctypes.c_int, [_vp, _dp, P(_i64)]),
        "vpm_set_time": (ctypes.c_int, [_vp, ctypes.c_double, _i64]),
        "vpm_set_particles": (ctypes.c_int, [_vp, _i64, _dp, _i64, _dp, _i64, _dp, _i64]),
        "vpm_append": (ctypes.c_int, [_vp, _i64, _dp, _i64, _dp, _i64, _dp, _i64, ctypes.c_int]),
        "vpm_truncate": (ctypes.c_int, [_vp, _i64]),
        "vpm_get_np": (ctypes.c_int, [_vp, P(_i64), P(_i64)]),
        "vpm_get_state": (ctypes.c_int, [_vp, _i64, _dp, _i64, _dp, _i64, _dp, _i64]),
        "vpm_get_sfs": (ctypes.c_int, [_vp, _i64, _dp, _i64, _dp, _i64]),
        "vpm_set_attributes": (ctypes.c_int, [_vp, _i64, _i64, _dp, _i64, _dp, _i64, _dp, _i64]),
        "vpm_get_attributes": (ctypes.c_int, [_vp, _i64, _i64, _dp, _i64, _dp, _i64,
                                              P(ctypes.c_int32)]),
        "vpm_eval_UJ": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
        "vpm_eval_UJ_targets": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _i64, _i64]),
        "vpm_get_UJ": (ctypes.c_int, [_vp, _i64, _i64, _dp, _i64, _dp, _i64]),
        "vpm_eval_sfs": (ctypes.c_int, [_vp, P(Scheme)]),
        "vpm_step": (ctypes.c_int, [_vp, ctypes.c_double, P(Scheme), _i64, ctypes.c_int]),
        "vpm_diagnostics": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp]),
        "vpm_centroids": (ctypes.c_int, [_vp, ctypes.c_int, P(_i64), P(_i64), _dp]),
        "vpm_fmm_default": (None, [P(Fmm)]),
        "vpm_eval_UJ_fmm": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, P(Fmm)]),
        "vpm_fmm_stats": (ctypes.c_int, [_vp, P(_i64)]),
        "vpm_save": (ctypes.c_int, [_vp, ctypes.c_char_p, _i64]),
        "vpm_load": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int]),
        "vpm_ffv_direct": (ctypes.c_int, [_vp, ctypes.c_int, _i64, _dp, _i64, _dp, _i64, _dp, _i64,
                                          _dp, _i64]),
        "vpm_uj_device_async": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _i64, _vp, _vp, _vp,
                                               _i64, _i64, _vp, _i64, _vp, _vp, _i64, _vp]),
        "vpm_uj_device_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _i64, _vp, _vp, _vp,
                                                 _i64, _i64, _vp, _i64, _vp, _vp, _i64, _vp]),
        "vpm_batch_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, P(_i64), P(_vp)]),
        "vpm_batch_destroy": (ctypes.c_int, [_vp]),
        "vpm_batch_last_error": (ctypes.c_int, [_vp, ctypes.c_char_p, _i64]),
        "vpm_batch_set_stream": (ctypes.c_int, [_vp, _vp]),
        "vpm_batch_set_field": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _i64, _dp, _i64, _dp,
                                               _i64]),
        "vpm_batch_get_field": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _i64, _dp, _i64, _dp,
                                               _i64]),
        "vpm_batch_eval_UJ": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
        "vpm_batch_get_UJ": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _i64, _dp, _i64]),
        "vpm_batch_step": (ctypes.c_int, [_vp, ctypes.c_double, P(Scheme), _i64, ctypes.c_int]),
        "vpm_batch_autotune": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp]),
        "vpm_batch_get_shapes": (ctypes.c_int, [_vp, P(ctypes.c_int32), P(ctypes.c_int32)]),
        "vpm_autotune": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, P(Tile), _dp]),
        "vpm_set_tile": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, P(Tile)]),
        "vpm_set_particle_order": (ctypes.c_int, [_vp, ctypes.c_int]),
        "vpm_batch_set_particle_order": (ctypes.c_int, [_vp, ctypes.c_int]),
        "vpm_measure_fma_peaks": (ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp]),
        "vpm_debug_fail_after": (ctypes.c_int, [_vp, _i64]),
        "vpm_debug_last_plan": (ctypes.c_int, [P(ctypes.c_int32), P(ctypes.c_int32),
                                               P(ctypes.c_int32), P(ctypes.c_int32)]),
        "vpm_get_launch_count": (ctypes.c_int, [_vp, P(_i64)]),
        "vpm_build_info": (ctypes.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def lib(build_if_missing: bool = True):
    """The loaded libvpmgpu.so (built in-tree on first use when nvcc exists)."""
    global _lib
    if _lib is None:
        if build_if_missing:
            from . import build as _build
            try:
                _build.build()
            except RuntimeError:
                if not os.path.exists(LIB_PATH):
                    raise
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libvpmgpu.so is not built ({LIB_PATH}); run "
                              "flowunsteady_gb300/build.py with the CUDA toolkit")
        _lib = _declare(ctypes.CDLL(LIB_PATH))
    return _lib


def last_error(ctx=None) -> str:
    buf = ctypes.create_string_buffer(512)
    lib().vpm_last_error(ctx, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, ctx=None):
    if rc != OK:
        raise VPMError(rc, last_error(ctx))


def dptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64, a.dtype
    return a.ctypes.data_as(_dp)


def default_scheme() -> Scheme:
    s = Scheme()
    lib().vpm_scheme_default(ctypes.byref(s))
    return s
