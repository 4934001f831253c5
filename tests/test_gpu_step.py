"""GPU time stepping (rVPM RHS, low-storage RK3 / Euler, core spreading,
dynamic SFS, clipping) against the CPU FP64 oracle, through the C ABI."""
import ctypes

import numpy as np
import pytest

from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300.workloads import leapfrog_rings, uniform_box
from tests.helpers import Ctx, rel_max, scheme

pytestmark = pytest.mark.gpu


def small_field(n=400, seed=80):
    X, G, S = uniform_box(n, seed_index=seed)
    return X * 0.5, G * 200.0, S * 3.0


@pytest.mark.parametrize("integ", [L.INTEGRATION_RK3, L.INTEGRATION_EULER])
@pytest.mark.parametrize("k,nu", [(L.KERNEL_WINCKELMANS, 0.0), (L.KERNEL_GAUSSIANERF, 1e-3)])
def test_step_fp64_matches_oracle(oracle, integ, k, nu):
    X, G, S = small_field()
    sc = scheme(kernel=k, prec=L.PREC_FP64, integration=integ, nu=nu, uinf=(0.1, 0, 0))
    Xo, Go, So, _, _ = oracle.step(sc, X, G, S, None, 0.01, nsteps=3)
    with Ctx(500) as c:
        c.set(X, G, S)
        c.step(sc, 0.01, nsteps=3)
        Xg, Gg, Sg = c.state()
    assert rel_max(Xg, Xo) <= 1e-13 and rel_max(Gg, Go) <= 1e-11 and rel_max(Sg, So) <= 1e-13


def test_step_dynamic_sfs_fp64_matches_oracle(oracle):
    X, G, S = small_field(300, 81)
    sc = scheme(kernel=1, prec=L.PREC_FP64, sfs=L.SFS_DYNAMIC,
                flags=L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE, rlxf=0.5, nu=1e-4)
    Xo, Go, So, Co, Eo = oracle.step(sc, X, G, S, None, 0.01, nsteps=2)
    with Ctx(300) as c:
        c.set(X, G, S)
        c.step(sc, 0.01, nsteps=2)
        Xg, Gg, Sg = c.state()
        Cg, Eg = c.sfs()
    assert rel_max(Xg, Xo) <= 1e-12 and rel_max(Gg, Go) <= 1e-9 and rel_max(Sg, So) <= 1e-12
    assert rel_max(Cg, Co) <= 1e-7
    assert rel_max(Eg, Eo) <= 1e-9
    assert np.any(Co[:, 0] != 0)


def test_graph_replay_equals_direct_launches():
    X, G, S = small_field(700, 82)
    sc = scheme(kernel=1, prec=L.PREC_FP32C, sfs=L.SFS_DYNAMIC, nu=1e-4)
    out = []
    for graph in (True, False):
        with Ctx(700) as c:
            c.set(X, G, S)
            c.step(sc, 0.005, nsteps=4, graph=graph)
            out.append(c.state())
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def test_static_particles_are_sources_only(oracle):
    X, G, S = small_field(200, 83)
    sc = scheme(kernel=1, prec=L.PREC_FP64)
    with Ctx(260) as c:
        c.set(X[:150], G[:150], S[:150])
        c.append(X[150:], G[150:], S[150:], static=True)
        c.step(sc, 0.01)
        Xg, Gg, Sg = c.state()
    assert np.array_equal(Xg[150:], X[150:]) and np.array_equal(Gg[150:], G[150:])
    Xo, Go, So, _, _ = oracle.step(sc, X, G, S, None, 0.01, n_static=50)
    assert rel_max(Xg, Xo) <= 1e-13 and rel_max(Gg, Go) <= 1e-11


def test_nonfinite_state_is_reported():
    X, G, S = small_field(64, 84)
    G[0] = 1e300
    with Ctx(64) as c:
        c.set(X, G, S)
        rc = c.lib.vpm_step(c.p, 1.0, ctypes.byref(scheme(kernel=0, prec=0)), 1, 0)
        assert rc == L.ERR_NONFINITE
        assert "non-finite" in L.last_error(c.p)


def test_fault_injection_hook():
    X, G, S = small_field(64, 85)
    with Ctx(64) as c:
        c.set(X, G, S)
        c.rc(c.lib.vpm_debug_fail_after(c.p, 1))
        assert c.lib.vpm_eval_UJ(c.p, 0, 0) == L.ERR_INJECTED
        Xg, _, _ = c.state()
        assert np.array_equal(Xg, X)
        c.uj(0, 0)  # hook disarmed after firing


def test_input_validation():
    X, G, S = small_field(10, 86)
    with Ctx(10) as c:
        bad = S.copy()
        bad[3] = -1.0
        for args, code in [((X, G, bad), L.ERR_INVALID)]:
            Xa, Ga, Sa = (np.ascontiguousarray(a) for a in args)
            rc = c.lib.vpm_set_particles(c.p, 10, L.dptr(Xa), 3, L.dptr(Ga), 3, L.dptr(Sa), 1)
            assert rc == code
        Xn = X.copy()
        Xn[2, 1] = np.nan
        assert c.lib.vpm_set_particles(c.p, 10, L.dptr(Xn), 3, L.dptr(G), 3, L.dptr(S), 1) == L.ERR_NONFINITE
        X11 = np.zeros((11, 3))
        assert c.lib.vpm_set_particles(c.p, 11, L.dptr(X11), 3, L.dptr(X11), 3,
                                       L.dptr(np.ones(11)), 1) == L.ERR_CAPACITY
        # core spreading needs the Gaussian kernel
        c.set(X, G, S)
        sc = scheme(kernel=0, nu=1e-3)
        assert c.lib.vpm_step(c.p, 0.01, ctypes.byref(sc), 1, 1) == L.ERR_UNSUPPORTED


def test_ring_diagnostics_match_oracle(oracle):
    X, G, S = leapfrog_rings(nstations=60)
    sc = scheme(kernel=1, prec=L.PREC_FP64, nu=1e-4)
    Xo, Go, So, _, _ = oracle.step(sc, X, G, S, None, 0.005, nsteps=2)
    d0 = oracle.diagnostics(1, Xo, Go, So)
    with Ctx(X.shape[0]) as c:
        c.set(X, G, S)
        c.step(sc, 0.005, nsteps=2)
        d = c.diag(1, L.PREC_FP64)
        n = X.shape[0] // 2
        st = (ctypes.c_int64 * 2)(0, n)
        en = (ctypes.c_int64 * 2)(n, 2 * n)
        cen = np.zeros((2, 3))
        c.rc(c.lib.vpm_centroids(c.p, 2, st, en, L.dptr(cen)))
    assert abs(d[0] - d0[0]) <= 1e-11 * abs(d0[0])
    assert np.allclose(d[1:4], d0[1:4], rtol=1e-11)
    w = np.linalg.norm(Go, axis=1)
    ref = np.array([(w[:n, None] * Xo[:n]).sum(0) / w[:n].sum(),
                    (w[n:, None] * Xo[n:]).sum(0) / w[n:].sum()])
    assert np.allclose(cen, ref, rtol=0, atol=1e-13)


@pytest.mark.parametrize("k", [L.KERNEL_WINCKELMANS, L.KERNEL_GAUSSIANERF])
def test_step_analytic_dynamic_sfs_matches_oracle(oracle, k):
    X, G, S = small_field(300, 87)
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE | L.SFS_ANALYTIC_DSIGMA
    sc = scheme(kernel=k, prec=L.PREC_FP64, sfs=L.SFS_DYNAMIC, flags=flags, rlxf=0.5,
                nu=1e-4 if k == L.KERNEL_GAUSSIANERF else 0.0)
    Xo, Go, So, Co, Eo = oracle.step(sc, X, G, S, None, 0.01, nsteps=2)
    with Ctx(300) as c:
        c.set(X, G, S)
        c.step(sc, 0.01, nsteps=2)
        Xg, Gg, Sg = c.state()
        Cg, Eg = c.sfs()
        assert rel_max(Xg, Xo) <= 1e-12 and rel_max(Gg, Go) <= 1e-10 and rel_max(Sg, So) <= 1e-12
        assert rel_max(Cg, Co) <= 1e-9 and rel_max(Eg, Eo) <= 1e-10
        # FP32C pair passes: the analytic α-derivatives keep C_d close to FP64.
        sc.precision = L.PREC_FP32C
        c.set(X, G, S)
        c.step(sc, 0.01, nsteps=2)
        C32, _ = c.sfs()
        m = (Co[:, 0] != 0) & (C32[:, 0] != 0)
        assert m.sum() > 50
        assert np.median(np.abs(C32[m, 0] - Co[m, 0]) / np.abs(Co[m, 0])) < 1e-4
