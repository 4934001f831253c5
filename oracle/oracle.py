"""ctypes front end of the CPU FP64 oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm as the checker.  The product
(flowunsteady_gb300, libvpmgpu.so) never imports it.

PARITY UNPINNED: FLOWVPM (the Julia package that holds the reference
arithmetic) is not vendored with FLOWUnsteady and Julia is absent, so the
oracle restates the published mathematics (docs/src/theory/rvpm.md:88-297 of
FLOWUnsteady) and is pinned against analytic known answers and an independent
NumPy restatement (oracle/np_oracle.py).  See vpm_oracle.cpp for every cite.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_lib = None

WINCKELMANS = 0
GAUSSIANERF = 1
# Length of the diagnostics vector (the VPM_DIAG_* layout of include/vpm_gpu.h).
DIAG_COUNT = 16

_dp = ctypes.POINTER(ctypes.c_double)
_i64 = ctypes.c_int64


def _elf_matches_host(path: str) -> bool:
    import platform
    want = {"x86_64": 0x3E, "aarch64": 0xB7, "arm64": 0xB7}.get(platform.machine())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if len(head) < 20 or head[:4] != b"\x7fELF":
        return False
    return want is None or int.from_bytes(head[18:20], "little") == want


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (g++ + OpenMP)."""
    src = os.path.join(_HERE, "vpm_oracle.cpp")
    stale = (not os.path.exists(_LIB) or not _elf_matches_host(_LIB)
             or os.path.getmtime(_LIB) < os.path.getmtime(src))
    if force or stale:
        subprocess.check_call(["make", "-s", "-B", "-C", _HERE, "liboracle.so"])
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB)
        _lib.orc_uj_direct.argtypes = [ctypes.c_int, ctypes.c_double, _i64, _dp, _i64, _dp, _dp,
                                       _dp, _dp, _dp, ctypes.c_int]
        _lib.orc_estr_direct.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, _i64, _dp,
                                         _dp, _dp, _i64, _dp, _dp, _dp, _dp, _dp, _dp, ctypes.c_int]
        _lib.orc_kernel_eval.argtypes = [ctypes.c_int, _i64, _dp, _dp, _dp, _dp]
        _lib.orc_step.argtypes = [ctypes.c_void_p, _i64, _i64, ctypes.c_double, _dp, _dp, _dp,
                                  _dp, _dp, ctypes.c_int]
        _lib.orc_diagnostics.argtypes = [ctypes.c_int, _i64, _i64, _dp, _dp, _dp, _dp, _dp,
                                         ctypes.c_int]
        _lib.orc_relax_pedrizzetti.argtypes = [_i64, ctypes.c_double, _dp, _dp]
        _lib.orc_uj_direct_dsigma.argtypes = [ctypes.c_int, _i64, _dp, _i64, _dp, _dp, _dp, _dp,
                                              ctypes.c_int]
        _lib.orc_ffv_direct.argtypes = [ctypes.c_int, _i64, _dp, _dp, _dp, _i64, _dp, _dp, _dp,
                                         ctypes.c_int]
        _lib.orc_estr_direct_dsigma.argtypes = [ctypes.c_int, ctypes.c_int, _i64, _dp, _dp, _dp,
                                                _dp, _dp, _dp, ctypes.c_int]
        _lib.orc_max_threads.restype = ctypes.c_int
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _c(a, shape_tail):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.reshape((-1,) + shape_tail) if shape_tail else a.reshape(-1)


def max_threads() -> int:
    return int(lib().orc_max_threads())


def kernel_eval(kernel: int, rho):
    rho = _c(rho, ())
    g, dg, z = (np.empty_like(rho) for _ in range(3))
    lib().orc_kernel_eval(kernel, rho.size, _p(rho), _p(g), _p(dg), _p(z))
    return g, dg, z


def uj_direct(kernel, X, G, S, Xt=None, sigma_scale=1.0, nthreads=0):
    """U (nt,3) and J (nt,3,3) at targets Xt (default: the sources)."""
    X, G, S = _c(X, (3,)), _c(G, (3,)), _c(S, ())
    Xt = X if Xt is None else _c(Xt, (3,))
    nt = Xt.shape[0]
    U = np.empty((nt, 3))
    J = np.empty((nt, 3, 3))
    lib().orc_uj_direct(kernel, sigma_scale, nt, _p(Xt), X.shape[0], _p(X), _p(G), _p(S), _p(U),
                        _p(J), nthreads)
    return U, J


def estr_direct(kernel, X, G, S, J, transposed=True, sigma_scale=1.0, nthreads=0):
    """E_str (n,3) and filtered vorticity ω (n,3) with targets = sources."""
    X, G, S = _c(X, (3,)), _c(G, (3,)), _c(S, ())
    J = None if J is None else _c(J, (3, 3))
    n = X.shape[0]
    E = np.empty((n, 3))
    om = np.empty((n, 3))
    lib().orc_estr_direct(kernel, sigma_scale, int(transposed), n, _p(X), _p(J), _p(S), n, _p(X),
                          _p(G), _p(S), _p(J), _p(E) if J is not None else None, _p(om), nthreads)
    return (E if J is not None else None), om


def estr_at(kernel, X, G, S, J, idx, transposed=True, sigma_scale=1.0, nthreads=0):
    """E_str (m,3) at the particles `idx` of the field (X, G, S), from J (n,3,3)
    at every particle (the targets' J is J[idx]); ζ uses the source core σ·scale."""
    X, G, S = _c(X, (3,)), _c(G, (3,)), _c(S, ())
    J = _c(J, (3, 3))
    idx = np.asarray(idx, dtype=np.int64)
    Xt = np.ascontiguousarray(X[idx])
    Jt = np.ascontiguousarray(J[idx])
    E = np.empty((idx.size, 3))
    lib().orc_estr_direct(kernel, sigma_scale, int(transposed), idx.size, _p(Xt), _p(Jt), None,
                          X.shape[0], _p(X), _p(G), _p(S), _p(J), _p(E), None, nthreads)
    return E


def zeta0(kernel) -> float:
    """ζ(0) of the kernel (the normalisation of the dynamic SFS denominator)."""
    return float(kernel_eval(kernel, np.zeros(1))[2][0])


def uj_dsigma(kernel, X, G, S, Xt=None, nthreads=0):
    """dJ/dα (nt,3,3) for core sizes ασ at α = 1."""
    X, G, S = _c(X, (3,)), _c(G, (3,)), _c(S, ())
    Xt = X if Xt is None else _c(Xt, (3,))
    DJ = np.empty((Xt.shape[0], 3, 3))
    lib().orc_uj_direct_dsigma(kernel, Xt.shape[0], _p(Xt), X.shape[0], _p(X), _p(G), _p(S),
                               _p(DJ), nthreads)
    return DJ


def estr_dsigma(kernel, X, G, S, J, DJ, transposed=True, nthreads=0):
    """dE_str/dα (n,3) at α = 1 (targets = sources)."""
    X, G, S = _c(X, (3,)), _c(G, (3,)), _c(S, ())
    J, DJ = _c(J, (3, 3)), _c(DJ, (3, 3))
    DE = np.empty((X.shape[0], 3))
    lib().orc_estr_direct_dsigma(kernel, int(transposed), X.shape[0], _p(X), _p(G), _p(S), _p(J),
                                 _p(DJ), _p(DE), nthreads)
    return DE


def ffv_direct(kernel, Xb, Gb, Sb, Xf, Gf, nthreads=0):
    """Free-vortex force terms M (nb, 6) of bound particles from free particles."""
    Xb, Gb, Sb = _c(Xb, (3,)), _c(Gb, (3,)), _c(Sb, ())
    Xf, Gf = _c(Xf, (3,)), _c(Gf, (3,))
    M = np.empty((Xb.shape[0], 6))
    lib().orc_ffv_direct(kernel, Xb.shape[0], _p(Xb), _p(Gb), _p(Sb), Xf.shape[0], _p(Xf), _p(Gf),
                         _p(M), nthreads)
    return M


def step(scheme_struct, X, G, S, C, dt, n_static=0, nsteps=1, nthreads=0):
    """Advance copies of the state by nsteps; returns (X, G, S, C, E_last)."""
    X, G, S = _c(X, (3,)).copy(), _c(G, (3,)).copy(), _c(S, ()).copy()
    n = X.shape[0]
    C = np.zeros((n, 3)) if C is None else _c(C, (3,)).copy()
    E = np.zeros((n, 3))
    for _ in range(nsteps):
        rc = lib().orc_step(ctypes.byref(scheme_struct), n, n_static, dt, _p(X), _p(G), _p(S),
                            _p(C), _p(E), nthreads)
        if rc != 0:
            raise RuntimeError(f"orc_step failed: {rc}")
    return X, G, S, C, E


def relax_pedrizzetti(G, J, rlx, nfree=None):
    G = _c(G, (3,)).copy()
    J = _c(J, (3, 3))
    nf = G.shape[0] if nfree is None else nfree
    lib().orc_relax_pedrizzetti(nf, rlx, _p(J), _p(G))
    return G


def diagnostics(kernel, X, G, S, C=None, n_static=0, nthreads=0):
    X, G, S = _c(X, (3,)), _c(G, (3,)), _c(S, ())
    C = None if C is None else _c(C, (3,))
    out = np.zeros(DIAG_COUNT)
    lib().orc_diagnostics(kernel, X.shape[0], n_static, _p(X), _p(G), _p(S), _p(C), _p(out),
                          nthreads)
    return out
