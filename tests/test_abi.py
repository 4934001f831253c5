"""CPU checks of the C ABI: the library builds and loads, exports every symbol
include/vpm_gpu.h declares, and rejects bad calls without a GPU."""
import ctypes
import os
import re

import numpy as np

from flowunsteady_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "vpm_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vpm_[a-zA-Z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = L.lib()
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(L.EXPORTS) == names


def test_build_info_names_sm103a():
    assert b"sm_103a" in L.lib().vpm_build_info()


def test_scheme_defaults():
    s = L.default_scheme()
    assert s.kernel == L.KERNEL_GAUSSIANERF and s.precision == L.PREC_FP32C
    assert s.integration == L.INTEGRATION_RK3 and s.transposed == 1
    assert s.f == 0.0 and abs(s.g - 0.2) < 1e-15 and s.sfs_alpha == 0.999
    # the struct's tail (treecode selection) lines up with the C layout
    assert s.uj_method == L.UJ_DIRECT and (s.fmm.p, s.fmm.ncrit, s.fmm.theta) == (4, 50, 0.4)
    assert s.fmm.sigma_factor == 7.1


def test_bad_calls_are_rejected_without_launch():
    lib = L.lib()
    assert lib.vpm_ctx_create(0, 0, None) == L.ERR_INVALID
    p = ctypes.c_void_p()
    assert lib.vpm_ctx_create(0, -5, ctypes.byref(p)) == L.ERR_INVALID
    assert lib.vpm_set_particles(None, 1, None, 3, None, 3, None, 1) == L.ERR_INVALID
    assert lib.vpm_eval_UJ(None, 0, 0) == L.ERR_INVALID
    assert lib.vpm_step(None, 0.1, None, 1, 1) == L.ERR_INVALID
    assert lib.vpm_set_particle_order(None, L.ORDER_CALLER) == L.ERR_INVALID
    assert lib.vpm_batch_set_particle_order(None, L.ORDER_AUTO) == L.ERR_INVALID
    x = np.zeros(3)
    assert lib.vpm_uj_device_async(7, 0, 1, None, None, None, 1, 1, None, 1, None, None, 1,
                                   None) == L.ERR_INVALID
    assert lib.vpm_uj_device_async(0, 9, 1, None, None, None, 1, 1, None, 1, None, None, 1,
                                   None) == L.ERR_INVALID
    n = (ctypes.c_int64 * 1)(-1)
    b = ctypes.c_void_p()
    assert lib.vpm_batch_create(0, 1, n, ctypes.byref(b)) == L.ERR_INVALID
    assert "field" in L.last_error() or L.last_error()
    del x


def test_header_enums_match_python_constants():
    src = open(os.path.join(ROOT, "include", "vpm_gpu.h")).read()
    for name, val in [("VPM_ERR_INVALID", L.ERR_INVALID), ("VPM_ERR_CAPACITY", L.ERR_CAPACITY),
                      ("VPM_ERR_NONFINITE", L.ERR_NONFINITE), ("VPM_ERR_INJECTED", L.ERR_INJECTED),
                      ("VPM_KERNEL_GAUSSIANERF", L.KERNEL_GAUSSIANERF),
                      ("VPM_PREC_FP32C", L.PREC_FP32C), ("VPM_DIAG_COUNT", L.DIAG_COUNT),
                      ("VPM_ORDER_AUTO", L.ORDER_AUTO), ("VPM_ORDER_CALLER", L.ORDER_CALLER)]:
        m = re.search(rf"{name}\s*=\s*(-?\d+)", src)
        assert m and int(m.group(1)) == val, name
