"""The particle field's bookkeeping on the GPU, through the C ABI and the
FLOWVPM-shaped Python API:

  - static (source-only) particles anywhere in the field: free particles may
    follow static ones, as FLOWUnsteady appends probes after the static
    particles of Vvpm_on_Xs (src/FLOWUnsteady_simulation.jl:516-541); a step
    of such a field equals the oracle's step of the same particles with the
    static ones moved to the tail (FP64 within 1e-12), and truncation
    restores the counts;
  - probes are plain particles with Γ = 0, σ = 1e-6 and vol = 0 (:572);
  - the shedding add_particle of FLOWUnsteady (:455-489): Γ = γ·V·dt·infD with
    the 5·eps floor, circulation max(|γ|, 5·eps), p_per_step particles along l;
  - vpm.monitor_Cd's statistics (src/FLOWUnsteady_monitors.jl:697-703),
    skewness and excess kurtosis included, against NumPy on the C_d column."""
import ctypes

import numpy as np
import pytest

from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300 import vpm
from flowunsteady_gb300.workloads import uniform_box
from tests.helpers import Ctx, rel_max, scheme

pytestmark = pytest.mark.gpu


def field(n, seed):
    X, G, S = uniform_box(n, seed_index=seed)
    return X * 0.5, G * 200.0, S * 3.0


def counts(c):
    n, ns = ctypes.c_int64(), ctypes.c_int64()
    c.rc(c.lib.vpm_get_np(c.p, ctypes.byref(n), ctypes.byref(ns)))
    return n.value, ns.value


@pytest.mark.parametrize("graph", [True, False])
def test_free_particles_after_static_ones_step_like_the_oracle(oracle, graph):
    X, G, S = field(260, 160)
    A, B, C = slice(0, 150), slice(150, 200), slice(200, 260)   # free, static, free
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE | L.SFS_ANALYTIC_DSIGMA
    sc = scheme(kernel=1, prec=L.PREC_FP64, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4)
    order = np.r_[np.arange(150), np.arange(200, 260), np.arange(150, 200)]
    Xo, Go, So, Co, _ = oracle.step(sc, X[order], G[order], S[order], None, 0.01, n_static=50,
                                    nsteps=2)
    inv = np.argsort(order)
    with Ctx(300) as c:
        c.set(X[A], G[A], S[A])
        c.append(X[B], G[B], S[B], static=True)
        c.append(X[C], G[C], S[C])
        assert counts(c) == (260, 50)
        c.step(sc, 0.01, nsteps=2, graph=graph)
        Xg, Gg, Sg = c.state()
        Cg, _ = c.sfs()
        d = c.diag(1, L.PREC_FP64)
    assert np.array_equal(Xg[B], X[B]) and np.array_equal(Gg[B], G[B])
    assert np.all(Cg[B] == 0.0)
    assert rel_max(Xg, Xo[inv]) <= 1e-12 and rel_max(Gg, Go[inv]) <= 1e-9
    assert rel_max(Sg, So[inv]) <= 1e-12 and rel_max(Cg[:, 0], Co[inv, 0]) <= 1e-7
    d0 = oracle.diagnostics(1, Xo, Go, So, Co, n_static=50)
    for k in (L.DIAG_NAMES.index(x) for x in ("cd_mean", "cd_std", "cd_zero_ratio", "cd_min",
                                               "cd_max")):
        assert abs(d[k] - d0[k]) <= 1e-7 * max(abs(d0[k]), 1e-3), L.DIAG_NAMES[k]


def test_truncate_restores_counts_and_the_tail_layout(oracle):
    X, G, S = field(200, 161)
    sc = scheme(kernel=1, prec=L.PREC_FP64)
    with Ctx(260) as c:
        c.set(X[:150], G[:150], S[:150])
        c.append(X[150:], G[150:], S[150:], static=True)
        c.append(np.zeros((7, 3)), np.zeros((7, 3)), np.full(7, 1e-6))     # probes: free
        assert counts(c) == (207, 50)
        c.rc(c.lib.vpm_truncate(c.p, 203))
        assert counts(c) == (203, 50)
        c.rc(c.lib.vpm_truncate(c.p, 200))
        assert counts(c) == (200, 50)
        c.rc(c.lib.vpm_truncate(c.p, 180))
        assert counts(c) == (180, 30)
        c.step(sc, 0.01)
        Xg, Gg, _ = c.state()
    Xo, Go, _, _, _ = oracle.step(sc, X[:180], G[:180], S[:180], None, 0.01, n_static=30)
    assert rel_max(Xg, Xo) <= 1e-13 and rel_max(Gg, Go) <= 1e-11


def test_probes_are_plain_particles_after_the_static_ones():
    X, G, S = field(300, 162)
    pf = vpm.ParticleField(400, kernel=vpm.gaussianerf, UJ=vpm.UJ_direct)
    vpm.add_particle(pf, X[:250], G[:250], S[:250])
    vpm.add_particle(pf, X[250:], G[250:], S[250:], static=True, vol=1e-3, circulation=0.5)
    P = np.array([[0.1, 0.2, 0.3], [0.3, -0.2, 0.0]])
    vpm.add_probe(pf, P)
    vol, circ, st = pf.attributes()
    assert pf.get_np() == 302 and pf.get_nstatic() == 50
    assert not st[300:].any() and st[250:300].all() and not st[:250].any()
    assert np.all(vol[300:] == 0.0) and np.all(vol[250:300] == 1e-3)
    assert np.all(circ[250:300] == 0.5) and np.all(circ[:250] == 1.0)
    Xg, Gg, Sg = pf.state()
    assert np.all(Gg[300:] == 0.0) and np.all(Sg[300:] == 1e-6)
    vpm.remove_particle(pf, 301)
    vpm.remove_particle(pf, 300)
    Up = vpm.Vvpm_on_Xs(pf, P)
    assert pf.get_np() == 300
    with Ctx(302) as c:
        c.set(np.vstack([X, P]), np.vstack([G, np.zeros((2, 3))]), np.r_[S, [1e-6, 1e-6]])
        Ur, _ = c.uj(1, L.PREC_FP64, 300, 302)
    assert rel_max(Up, Ur) <= 1e-12
    pf.close()


def test_shed_particles_follow_flowunsteady_add_particle():
    pf = vpm.ParticleField(64)
    X = np.array([0.1, 0.0, -0.2])
    l = np.array([0.0, 0.4, 0.0])
    infD = np.array([0.0, 1.0, 0.0])
    vpm.add_shed_particles(pf, X, 2.5, 0.01, 3.0, infD, 0.08, 2e-4, l, 4)
    # An empty sheet: |Γ| below 5·eps is raised to 5·eps per component.
    vpm.add_shed_particles(pf, X, 0.0, 0.01, 3.0, infD, 0.08, 2e-4, l, 2, overwrite_sigma=0.03)
    Xg, Gg, Sg = pf.state()
    vol, circ, _ = pf.attributes()
    eps = np.finfo(np.float64).eps
    i = np.arange(1, 5)[:, None]
    assert np.allclose(Xg[:4], X + i * l / 4 - l / 8, rtol=0, atol=1e-15)
    assert np.allclose(Gg[:4], 2.5 * 3.0 * 0.01 * infD / 4, rtol=1e-15, atol=0)
    assert np.allclose(Sg[:4], 0.02) and np.allclose(vol[:4], 5e-5) and np.all(circ[:4] == 2.5)
    assert np.allclose(Gg[4:], 5 * eps / 2) and np.all(Sg[4:] == 0.03)
    assert np.all(circ[4:] == 5 * eps)
    pf.close()


def test_monitor_cd_statistics_match_numpy():
    X, G, S = field(900, 163)
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_ANALYTIC_DSIGMA
    sc = scheme(kernel=1, prec=L.PREC_FP64, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4, maxC=0.0)
    with Ctx(950) as c:
        c.set(X[:850], G[:850], S[:850])
        c.append(X[850:], G[850:], S[850:], static=True)
        c.step(sc, 0.01)
        C, _ = c.sfs()
        d = dict(zip(L.DIAG_NAMES, c.diag(1, L.PREC_FP64)))
    cd = C[:850, 0]
    nz = cd[cd != 0.0]
    assert nz.size > 100 and np.any(nz < 0) and np.any(nz > 0)
    m = nz.mean()
    m2, m3, m4 = (((nz - m) ** k).mean() for k in (2, 3, 4))
    assert abs(d["cd_zero_ratio"] - (cd == 0).mean()) <= 1e-15
    assert abs(d["cd_mean"] - m) <= 1e-12 * abs(nz).max()
    assert abs(d["cd_std"] - np.sqrt(m2)) <= 1e-9 * np.sqrt(m2)
    assert abs(d["cd_skew"] - m3 / m2**1.5) <= 1e-7 * max(1.0, abs(m3 / m2**1.5))
    assert abs(d["cd_kurt"] - (m4 / m2**2 - 3.0)) <= 1e-7 * max(1.0, abs(m4 / m2**2))
    assert d["cd_min"] == nz.min() and d["cd_max"] == nz.max()
