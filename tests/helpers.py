import ctypes

import numpy as np

from flowunsteady_gb300 import _lib as L


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


def rel_max(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


class Ctx:
    """Thin C-ABI context used by the GPU tests (no Python-side logic)."""

    def __init__(self, cap, device=0):
        self.lib = L.lib()
        p = ctypes.c_void_p()
        L.check(self.lib.vpm_ctx_create(device, int(cap), ctypes.byref(p)))
        self.p = p

    def close(self):
        if self.p:
            self.lib.vpm_ctx_destroy(self.p)
            self.p = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def rc(self, rc):
        L.check(rc, self.p)

    def set(self, X, G, S):
        X = np.ascontiguousarray(X, np.float64)
        G = np.ascontiguousarray(G, np.float64)
        S = np.ascontiguousarray(S, np.float64)
        self.rc(self.lib.vpm_set_particles(self.p, X.shape[0], L.dptr(X), 3, L.dptr(G), 3,
                                           L.dptr(S), 1))

    def append(self, X, G, S, static=False):
        X = np.ascontiguousarray(X, np.float64)
        G = np.ascontiguousarray(G, np.float64)
        S = np.ascontiguousarray(S, np.float64)
        self.rc(self.lib.vpm_append(self.p, X.shape[0], L.dptr(X), 3, L.dptr(G), 3, L.dptr(S),
                                    1, 1 if static else 0))

    def uj(self, kernel, prec, t0=None, t1=None):
        n = self.np()
        if t0 is None:
            self.rc(self.lib.vpm_eval_UJ(self.p, kernel, prec))
            t0, t1 = 0, n
        else:
            self.rc(self.lib.vpm_eval_UJ_targets(self.p, kernel, prec, t0, t1))
        m = t1 - t0
        U, J = np.empty((m, 3)), np.empty((m, 3, 3))
        self.rc(self.lib.vpm_get_UJ(self.p, t0, m, L.dptr(U), 3, L.dptr(J), 9))
        return U, J

    def np(self):
        n, ns = ctypes.c_int64(), ctypes.c_int64()
        self.rc(self.lib.vpm_get_np(self.p, ctypes.byref(n), ctypes.byref(ns)))
        return n.value

    def state(self):
        n = self.np()
        X, G, S = np.empty((n, 3)), np.empty((n, 3)), np.empty(n)
        self.rc(self.lib.vpm_get_state(self.p, n, L.dptr(X), 3, L.dptr(G), 3, L.dptr(S), 1))
        return X, G, S

    def sfs(self):
        n = self.np()
        C, E = np.empty((n, 3)), np.empty((n, 3))
        self.rc(self.lib.vpm_get_sfs(self.p, n, L.dptr(C), 3, L.dptr(E), 3))
        return C, E

    def step(self, scheme, dt, nsteps=1, graph=True):
        self.rc(self.lib.vpm_step(self.p, dt, ctypes.byref(scheme), nsteps, 1 if graph else 0))

    def diag(self, kernel, prec):
        out = np.zeros(L.DIAG_COUNT)
        self.rc(self.lib.vpm_diagnostics(self.p, kernel, prec, L.dptr(out)))
        return out


def scheme(kernel=1, prec=0, integration=1, transposed=1, sfs=0, nu=0.0, f=0.0, g=0.2,
           flags=1, alpha=0.999, rlxf=1.0, minC=0.0, maxC=1.0, uinf=(0, 0, 0), Cd=0.0):
    s = L.Scheme()
    s.kernel, s.precision, s.integration, s.transposed = kernel, prec, integration, transposed
    s.f, s.g = f, g
    for k in range(3):
        s.uinf[k] = uinf[k]
    s.nu = nu
    s.sfs, s.sfs_flags = sfs, flags
    s.sfs_alpha, s.sfs_rlxf, s.sfs_minC, s.sfs_maxC = alpha, rlxf, minC, maxC
    s.sfs_Cd = Cd
    s.relaxation, s.relax_nsteps, s.relax_factor = 0, 1, 0.3
    return s
