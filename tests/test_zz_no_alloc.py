"""vpm_uj_device_noalloc: the U/∇U evaluation for callers that cannot let the
library allocate device memory (loops that must not allocate once running,
hosts whose own pool allocator holds the GPU's memory).  On every call it
must give what the CPU FP64 oracle gives (FP64 within 1e-12, FP32C within
1e-5 relative L2) and what vpm_uj_device_async gives on the same device
arrays, with its split-source scratch in a fixed array instead of an
allocation.

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
    return U.cpu().numpy().T, J.cpu().numpy().T.reshape(m, 3, 3)


def _plan():
    """(source chunks, cluster size) of the last stateless U/J call."""
    n_chunk, cluster = ctypes.c_int32(), ctypes.c_int32()
    L.lib().vpm_debug_last_plan(None, None, ctypes.byref(n_chunk), ctypes.byref(cluster))
    return n_chunk.value, cluster.value


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("kernel,prec,tol", [
    (L.KERNEL_GAUSSIANERF, L.PREC_FP64, 1e-12),
    (L.KERNEL_WINCKELMANS, L.PREC_FP32C, 1e-5),
    (L.KERNEL_GAUSSIANERF, L.PREC_FP32C, 1e-5),
])
def test_noalloc_matches_oracle_and_allocating_entry_point(oracle, kernel, prec, tol):
    torch = pytest.importorskip("torch")
    lib = L.lib()
    n = 6000
    X, G, S = uniform_box(n, seed_index=90)
    S = S * 2.0
    Xd, Gd, Sd = _dev(torch, X.T), _dev(torch, G.T), _dev(torch, S)
    # Targets: all particles (self pairs skipped) and a separate probe set.
    rng = np.random.default_rng(3)
    P = rng.uniform(-1, 1, (1000, 3))
    Xp = _dev(torch, P.T)
    split = []
    for m, Xt, pts in ((n, None, X), (1000, Xp, P)):
        U0, J0 = oracle.uj_direct(kernel, X, G, S, Xt=pts)
        Ua, Ja = _call(lib.vpm_uj_device_async, torch, kernel, prec, n, Xd, Gd, Sd, m, Xt)
        for _ in range(2):   # two calls in a row share the static scratch
            U1, J1 = _call(lib.vpm_uj_device_noalloc, torch, kernel, prec, n, Xd, Gd, Sd, m, Xt)
            split.append(_plan())
            assert _rel_l2(U1, U0) <= tol and _rel_l2(J1, J0) <= tol
            assert _rel_l2(U1, Ua) <= tol and _rel_l2(J1, Ja) <= tol
    # The source range was split in every call.  FP64 sums the chunks through
    # the static scratch; FP32C chunks may instead run as thread-block clusters
    # that sum in shared memory (then the scratch is not touched).
    assert all(nc > 1 for nc, _ in split)
    if prec == L.PREC_FP64:
        assert all(cl == 1 for _, cl in split)


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
