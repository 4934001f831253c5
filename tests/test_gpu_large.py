"""Parity at the sizes the throughput figures are quoted on, against the CPU
FP64 oracle on seeded target samples (the oracle cannot afford N² at these
sizes; each sample costs it seconds):

  - the 262,144-particle helical wake, both kernels: the full-field GPU FP64
    evaluation (Morton-ordered, with the Gaussian-erf far form from ρ² = 90)
    within 1e-12 relative L2 of the oracle, and the FP32C evaluation within
    1e-5, on 2,048 sampled targets;
  - the 1,048,576-particle 12-turn helical wake, Gaussian-erf: the FP32C
    evaluation within 1e-5 of the oracle on 4,096 sampled targets, and the
    GPU FP64 sum at those targets (target-subset form) within 1e-12;
  - E_str of an SFS evaluation of the 262,144-particle wake (FP64 within 1e-10,
    FP32C within 2e-4) and the dynamic C_d of the finite-difference procedure
    (FP64, within 1e-7) on the sampled particles.  E_str at a particle needs
    J at every source; the oracle takes it from the GPU FP64 evaluation, which
    the first test ties to the oracle.

Formulas: docs/src/theory/rvpm.md:88-99 (U, J), :251-262 (E_str), :264-294
(C_d) of FLOWUnsteady."""
import ctypes

import numpy as np
import pytest

from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300.workloads import helical_wake
from tests.helpers import Ctx, rel_l2, scheme

pytestmark = pytest.mark.gpu


def sample(n, m, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, m, replace=False))


def uj_at_targets(torch, kernel, prec, X, G, S, Xt):
    """GPU U/J of the sources (X, G, S) at the points Xt (vpm_uj_device_async)."""
    dev = torch.device("cuda:0")
    n, m = X.shape[0], Xt.shape[0]
    Xd = torch.tensor(np.ascontiguousarray(X.T), device=dev)
    Gd = torch.tensor(np.ascontiguousarray(G.T), device=dev)
    Sd = torch.tensor(np.ascontiguousarray(S), device=dev)
    Td = torch.tensor(np.ascontiguousarray(Xt.T), device=dev)
    Ud = torch.zeros((3, m), dtype=torch.float64, device=dev)
    Jd = torch.zeros((9, m), dtype=torch.float64, device=dev)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.lib().vpm_uj_device_async(kernel, prec, n, Xd.data_ptr(), Gd.data_ptr(), Sd.data_ptr(),
                                     n, m, Td.data_ptr(), m, Ud.data_ptr(), Jd.data_ptr(), m, st)
    assert rc == 0, L.last_error()
    torch.cuda.synchronize()
    return Ud.cpu().numpy().T.copy(), Jd.cpu().numpy().T.reshape(m, 3, 3).copy()


def stretch(J, G, transposed=True):
    return np.einsum("iba,ib->ia", J, G) if transposed else np.einsum("iab,ib->ia", J, G)


@pytest.mark.parametrize("k", [L.KERNEL_WINCKELMANS, L.KERNEL_GAUSSIANERF])
def test_helical_wake_262144_against_oracle(oracle, k):
    X, G, S = helical_wake(262144)
    idx = sample(X.shape[0], 2048, 200 + k)
    U0, J0 = oracle.uj_direct(k, X, G, S, Xt=X[idx])
    with Ctx(X.shape[0]) as c:
        c.set(X, G, S)
        U64, J64 = c.uj(k, L.PREC_FP64)
        U32, J32 = c.uj(k, L.PREC_FP32C)
    assert rel_l2(U64[idx], U0) <= 1e-12 and rel_l2(J64[idx], J0) <= 1e-12
    assert rel_l2(U32[idx], U0) <= 1e-5 and rel_l2(J32[idx], J0) <= 1e-5
    assert rel_l2(stretch(J32[idx], G[idx]), stretch(J0, G[idx])) <= 1e-5


def test_helical_wake_1048576_against_oracle(oracle):
    torch = pytest.importorskip("torch")
    k = L.KERNEL_GAUSSIANERF
    X, G, S = helical_wake(1048576, turns=12)
    idx = sample(X.shape[0], 4096, 210)
    U0, J0 = oracle.uj_direct(k, X, G, S, Xt=X[idx])
    with Ctx(X.shape[0]) as c:
        c.set(X, G, S)
        U32, J32 = c.uj(k, L.PREC_FP32C)
    assert rel_l2(U32[idx], U0) <= 1e-5 and rel_l2(J32[idx], J0) <= 1e-5
    U64, J64 = uj_at_targets(torch, k, L.PREC_FP64, X, G, S, X[idx])
    assert rel_l2(U64, U0) <= 1e-12 and rel_l2(J64, J0) <= 1e-12


def test_helical_wake_262144_sfs_against_oracle(oracle):
    k = L.KERNEL_GAUSSIANERF
    al = 0.999
    X, G, S = helical_wake(262144)
    n = X.shape[0]
    idx = sample(n, 1024, 220)
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE
    with Ctx(n) as c:
        c.set(X, G, S)
        # E_str of the SFS pass (constant C_d: no dynamic procedure) in FP32C.
        c.rc(c.lib.vpm_eval_sfs(c.p, ctypes.byref(
            scheme(kernel=k, prec=L.PREC_FP32C, sfs=L.SFS_CONSTANT, Cd=0.1))))
        _, E32 = c.sfs()
        # The dynamic procedure in FP64 (test filter at ασ).
        c.rc(c.lib.vpm_eval_sfs(c.p, ctypes.byref(
            scheme(kernel=k, prec=L.PREC_FP64, sfs=L.SFS_DYNAMIC, flags=flags, alpha=al))))
        C64, E64 = c.sfs()
        _, J = c.uj(k, L.PREC_FP64)
        c.set(X, G, S * al)
        _, Ja = c.uj(k, L.PREC_FP64)
    # The oracle's E_str at the sampled particles from every source's J.
    Eo = oracle.estr_at(k, X, G, S, J, idx)
    Eao = oracle.estr_at(k, X, G, S, Ja, idx, sigma_scale=al)
    assert rel_l2(E64[idx], Eo) <= 1e-10
    assert rel_l2(E32[idx], Eo) <= 2e-4
    # Dynamic C_d (pseudo-three-level, positive, backscatter clipping), restated
    # from the oracle's step at the sampled particles.
    Gi, Si = G[idx], S[idx]
    nume = (3 * al - 2) * np.einsum("ia,ia->i", Gi, stretch(Ja[idx], Gi) - stretch(J[idx], Gi))
    deno = Si**3 / oracle.zeta0(k) * np.einsum("ia,ia->i", Gi, Eao - Eo)
    cd = np.where(deno != 0, nume / np.where(deno != 0, deno, 1.0), 0.0)
    cd = np.minimum(np.abs(cd), 1.0)
    cd = np.where(cd * np.einsum("ia,ia->i", Gi, Eo) < 0, 0.0, cd)
    assert np.count_nonzero(cd) > 100
    assert rel_l2(C64[idx, 0], cd) <= 1e-7
