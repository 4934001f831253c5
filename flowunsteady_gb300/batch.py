"""Many independent particle fields advanced together (vpm_batch_* of the C ABI).

Each pair pass of a batch is one persistent launch over a flattened
(field, target tile, source chunk) queue; each time step is one CUDA-graph
replay.  Fields never interact.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np

from . import _lib as L


class FieldBatch:
    def __init__(self, sizes: Sequence[int], device: int = 0):
        self.sizes = [int(n) for n in sizes]
        arr = (ctypes.c_int64 * len(self.sizes))(*self.sizes)
        ptr = ctypes.c_void_p()
        rc = L.lib().vpm_batch_create(int(device), len(self.sizes), arr, ctypes.byref(ptr))
        if rc != L.OK:
            raise L.VPMError(rc, L.last_error())
        self._b = ptr

    def _check(self, rc):
        if rc != L.OK:
            buf = ctypes.create_string_buffer(512)
            L.lib().vpm_batch_last_error(self._b, buf, len(buf))
            raise L.VPMError(rc, buf.value.decode(errors="replace"))

    def close(self):
        if getattr(self, "_b", None):
            L.lib().vpm_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_particle_order(self, mode):
        """L.ORDER_AUTO (each field along its own Morton curve) or
        L.ORDER_CALLER (vpm_batch_set_particle_order)."""
        self._check(L.lib().vpm_batch_set_particle_order(self._b, int(mode)))

    def set_field(self, f, X, Gamma, sigma):
        X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, 3)
        G = np.ascontiguousarray(Gamma, dtype=np.float64).reshape(-1, 3)
        S = np.ascontiguousarray(sigma, dtype=np.float64).reshape(-1)
        self._check(L.lib().vpm_batch_set_field(self._b, f, L.dptr(X), 3, L.dptr(G), 3,
                                                L.dptr(S), 1))

    def get_field(self, f):
        n = self.sizes[f]
        X, G, S = np.empty((n, 3)), np.empty((n, 3)), np.empty(n)
        self._check(L.lib().vpm_batch_get_field(self._b, f, L.dptr(X), 3, L.dptr(G), 3,
                                                L.dptr(S), 1))
        return X, G, S

    def eval_UJ(self, kernel: int, precision: int):
        self._check(L.lib().vpm_batch_eval_UJ(self._b, kernel, precision))

    def get_UJ(self, f):
        n = self.sizes[f]
        U, J = np.empty((n, 3)), np.empty((n, 3, 3))
        self._check(L.lib().vpm_batch_get_UJ(self._b, f, L.dptr(U), 3, L.dptr(J), 9))
        return U, J

    def step(self, dt: float, scheme: "L.Scheme", nsteps: int = 1, use_graph: bool = True):
        self._check(L.lib().vpm_batch_step(self._b, float(dt), ctypes.byref(scheme), int(nsteps),
                                           1 if use_graph else 0))

    def autotune(self, kernel: int, precision: int) -> float:
        """Tile shape per size bucket (vpm_batch_autotune); returns the tuned
        batch's U/J pass time in ms."""
        ms = ctypes.c_double()
        self._check(L.lib().vpm_batch_autotune(self._b, kernel, precision, ctypes.byref(ms)))
        return ms.value

    def shapes(self):
        """(block, targets per thread) of every field in the current plan."""
        nf = len(self.sizes)
        blk, tpt = (ctypes.c_int32 * nf)(), (ctypes.c_int32 * nf)()
        self._check(L.lib().vpm_batch_get_shapes(self._b, blk, tpt))
        return list(zip(list(blk), list(tpt)))

    def set_stream(self, stream_handle: int):
        self._check(L.lib().vpm_batch_set_stream(self._b, ctypes.c_void_p(stream_handle)))
