"""vpm_uj_device_noalloc: the U/∇U evaluation for callers that cannot let the
library allocate device memory (fixed-memory loops, hosts whose pool
allocator owns the GPU's memory, work inside a graph capture).  It must give
what vpm_uj_device_async gives on the same device arrays, on every call, with
its scratch in a fixed array instead of an allocation.

This file is named to run last: a failure here leaves every other test run."""
import ctypes

import numpy as np
import pytest

from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300.workloads import uniform_box

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.tensor(np.ascontiguousarray(a), device="cuda:0")


def _call(fn, torch, kernel, prec, n, Xd, Gd, Sd, m, Xt):
    U = torch.zeros((3, m), dtype=torch.float64, device="cuda:0")
    J = torch.zeros((9, m), dtype=torch.float64, device="cuda:0")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = fn(kernel, prec, n, Xd.data_ptr(), Gd.data_ptr(), Sd.data_ptr(), n, m,
            None if Xt is None else Xt.data_ptr(), m, U.data_ptr(), J.data_ptr(), m, st)
    assert rc == 0, L.last_error()
    torch.cuda.synchronize()
    return U.cpu().numpy(), J.cpu().numpy()


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("kernel,prec,tol", [
    (L.KERNEL_GAUSSIANERF, L.PREC_FP64, 1e-12),
    (L.KERNEL_WINCKELMANS, L.PREC_FP32C, 1e-5),
    (L.KERNEL_GAUSSIANERF, L.PREC_FP32C, 1e-5),
])
def test_noalloc_matches_allocating_entry_point(kernel, prec, tol):
    torch = pytest.importorskip("torch")
    lib = L.lib()
    n = 6000
    X, G, S = uniform_box(n, seed_index=90)
    Xd, Gd, Sd = _dev(torch, X.T), _dev(torch, G.T), _dev(torch, S * 2.0)
    # Targets: all particles (self pairs skipped) and a separate probe set.
    rng = np.random.default_rng(3)
    Xp = _dev(torch, rng.uniform(-1, 1, (1000, 3)).T)
    for m, Xt in ((n, None), (1000, Xp)):
        U0, J0 = _call(lib.vpm_uj_device_async, torch, kernel, prec, n, Xd, Gd, Sd, m, Xt)
        for _ in range(2):   # two calls in a row share the static scratch
            U1, J1 = _call(lib.vpm_uj_device_noalloc, torch, kernel, prec, n, Xd, Gd, Sd, m, Xt)
            assert _rel_l2(U1, U0) <= tol and _rel_l2(J1, J0) <= tol


def test_noalloc_rejects_more_targets_than_its_scratch_holds():
    torch = pytest.importorskip("torch")
    lib = L.lib()
    n = 16385
    X, G, S = uniform_box(n, seed_index=91)
    Xd, Gd, Sd = _dev(torch, X.T), _dev(torch, G.T), _dev(torch, S)
    U = torch.zeros((3, n), dtype=torch.float64, device="cuda:0")
    J = torch.zeros((9, n), dtype=torch.float64, device="cuda:0")
    rc = lib.vpm_uj_device_noalloc(0, L.PREC_FP32C, n, Xd.data_ptr(), Gd.data_ptr(),
                                   Sd.data_ptr(), n, n, None, n, U.data_ptr(), J.data_ptr(), n,
                                   None)
    assert rc == L.ERR_CAPACITY
    assert "16384" in L.last_error()
    torch.cuda.synchronize()
    assert float(U.abs().max()) == 0.0
