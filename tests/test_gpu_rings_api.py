"""The leapfrogging-ring case (full scheme) against the oracle, Pedrizzetti
relaxation, the autotuner, coincident-pair semantics and the FLOWVPM-shaped
Python API, on the GPU through the C ABI."""
import ctypes

import numpy as np
import pytest

from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300 import vpm
from flowunsteady_gb300.workloads import leapfrog_rings, uniform_box
from tests.helpers import Ctx, rel_l2, rel_max, scheme

pytestmark = pytest.mark.gpu


def ring_scheme(prec):
    return scheme(kernel=L.KERNEL_GAUSSIANERF, prec=prec, sfs=L.SFS_DYNAMIC,
                  flags=L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE, nu=1e-4)


def test_leapfrog_rings_full_scheme_matches_oracle(oracle):
    # 7,600 particles, Gaussian-erf, transposed rVPM, dynamic SFS with clipping,
    # core spreading, RK3 dt = 0.005: 10 steps.
    X, G, S = leapfrog_rings()
    Xo, Go, So, Co, _ = oracle.step(ring_scheme(L.PREC_FP64), X, G, S, None, 0.005, nsteps=10)
    d0 = oracle.diagnostics(1, Xo, Go, So, Co)
    with Ctx(X.shape[0]) as c:
        c.set(X, G, S)
        c.step(ring_scheme(L.PREC_FP64), 0.005, nsteps=10)
        Xg, Gg, Sg = c.state()
        Cg, _ = c.sfs()
        d = c.diag(1, L.PREC_FP64)
    assert np.abs(Xg - Xo).max() <= 1e-12
    assert rel_l2(Gg, Go) <= 1e-10 and np.abs(Sg - So).max() <= 1e-13
    assert rel_l2(Cg[:, 0], Co[:, 0]) <= 1e-6
    assert abs(d[0] - d0[0]) <= 1e-10 * abs(d0[0]) and abs(d[3] - d0[3]) <= 1e-12 * abs(d0[3])
    # FP32C pair passes with the finite-difference C_d: the (α-1)^{-1} = 1000
    # amplification of FP32 noise in C_d shows in the trajectory.
    with Ctx(X.shape[0]) as c:
        c.set(X, G, S)
        c.step(ring_scheme(L.PREC_FP32C), 0.005, nsteps=10)
        X32, G32, S32 = c.state()
    assert np.abs(X32 - Xo).max() <= 1e-4 and rel_l2(G32, Go) <= 1e-3


def test_leapfrog_rings_analytic_sfs_fp32c_tracks_fp64(oracle):
    # With the analytic α-derivatives the FP32C trajectory stays at FP32 distance.
    X, G, S = leapfrog_rings()
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE | L.SFS_ANALYTIC_DSIGMA
    s64 = scheme(kernel=1, prec=L.PREC_FP64, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4)
    Xo, Go, So, Co, _ = oracle.step(s64, X, G, S, None, 0.005, nsteps=10)
    with Ctx(X.shape[0]) as c:
        c.set(X, G, S)
        c.step(s64, 0.005, nsteps=10)
        X64, G64, _ = c.state()
        assert np.abs(X64 - Xo).max() <= 1e-12 and rel_l2(G64, Go) <= 1e-10
        s32 = scheme(kernel=1, prec=L.PREC_FP32C, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4)
        c.set(X, G, S)
        c.step(s32, 0.005, nsteps=10)
        X32, G32, _ = c.state()
    assert np.abs(X32 - Xo).max() <= 1e-7 and rel_l2(G32, Go) <= 1e-6


def test_pedrizzetti_relaxation_matches_oracle(oracle):
    X, G, S = uniform_box(300, seed_index=120)
    X, G, S = X * 0.4, G * 100, S * 3
    sc = scheme(kernel=1, prec=L.PREC_FP64)
    sc.relaxation, sc.relax_nsteps, sc.relax_factor = L.RELAX_PEDRIZZETTI, 1, 0.3
    sc0 = scheme(kernel=1, prec=L.PREC_FP64)
    Xo, Go, So, _, _ = oracle.step(sc0, X, G, S, None, 0.01)
    _, J = oracle.uj_direct(1, Xo, Go, So)
    Gr = oracle.relax_pedrizzetti(Go, J, 0.3)
    with Ctx(300) as c:
        c.set(X, G, S)
        c.step(sc, 0.01)
        Xg, Gg, Sg = c.state()
    assert rel_max(Xg, Xo) <= 1e-13 and rel_max(Gg, Gr) <= 1e-10


def test_autotune_picks_a_compiled_shape_and_keeps_parity(oracle):
    X, G, S = uniform_box(5000, seed_index=121)
    U0, J0 = oracle.uj_direct(0, X, G, S)
    with Ctx(5000) as c:
        c.set(X, G, S)
        tile, ms = L.Tile(), ctypes.c_double()
        c.rc(c.lib.vpm_autotune(c.p, 0, L.PREC_FP32C, ctypes.byref(tile), ctypes.byref(ms)))
        assert (tile.block, tile.tpt) in {(128, 2), (128, 4), (256, 2)} and ms.value > 0
        # The ζ pass is tuned separately; its shape comes back packed.
        assert divmod(tile.reserved, 16) in {(128, 2), (128, 4), (256, 2)}
        U, J = c.uj(0, L.PREC_FP32C)
        assert rel_l2(U, U0) <= 1e-5 and rel_l2(J, J0) <= 1e-5
        bad = L.Tile(64, 3, 0, 0)
        assert c.lib.vpm_set_tile(c.p, 0, L.PREC_FP32C, ctypes.byref(bad)) == L.ERR_UNSUPPORTED


@pytest.mark.parametrize("k", [L.KERNEL_WINCKELMANS, L.KERNEL_GAUSSIANERF])
@pytest.mark.parametrize("n", [5000, 70000])
def test_coincident_distinct_particles_are_skipped(oracle, k, n):
    # Exact twins in distant source tiles (and, at n = 70,000, in the Morton
    # order of the sorted passes): every precision skips the coincident pair
    # in U/J and in the ζ pass behind E_str, as the oracle does
    # (src/FLOWUnsteady_processing_force.jl:895).  Checked row by row at the
    # twins, where an unskipped pair would add q(0)ε·Γ to J and ζ(0)Γ to Ω.
    X, G, S = uniform_box(n, seed_index=122)
    S = S * 2.0
    twins = [(0, n - 1), (1, n // 2), (7, 8)]
    for a, b in twins:
        X[b] = X[a]
    rows = np.array(sorted({i for t in twins for i in t}))
    U0, J0 = oracle.uj_direct(k, X, G, S, Xt=X[rows])
    sc = scheme(kernel=k, prec=L.PREC_FP64, sfs=L.SFS_CONSTANT, Cd=0.1, flags=0)
    with Ctx(n) as c:
        c.set(X, G, S)
        U64, J64 = c.uj(k, L.PREC_FP64)
        E0 = oracle.estr_at(k, X, G, S, J64, rows)
        for prec, tol in ((L.PREC_FP64, 1e-12), (L.PREC_FP32C, 1e-5), (L.PREC_FP32, 1e-3)):
            U, J = c.uj(k, prec)
            for r, i in enumerate(rows):
                assert rel_l2(U[i], U0[r]) <= tol and rel_l2(J[i], J0[r]) <= tol, (prec, i)
            sc.precision = prec
            c.rc(c.lib.vpm_eval_sfs(c.p, ctypes.byref(sc)))
            _, E = c.sfs()
            for r, i in enumerate(rows):
                assert rel_l2(E[i], E0[r]) <= 20 * tol, (prec, i)


def test_python_api_mirrors_flowvpm():
    X, G, S = uniform_box(800, seed_index=123)
    pf = vpm.ParticleField(1200, kernel=vpm.gaussianerf, UJ=vpm.UJ_direct,
                           SFS=vpm.DynamicSFS(alpha=0.999, maxC=1.0),
                           viscous=vpm.CoreSpreading(nu=1e-4))
    vpm.add_particle(pf, X[:500], G[:500], S[:500])
    for i in range(500, 800):
        vpm.add_particle(pf, X[i], G[i], S[i])
    assert vpm.get_np(pf) == 800
    pf.UJ(pf)
    U, J = pf.get_UJ()
    assert U.shape == (800, 3) and J.shape == (800, 3, 3)
    probes = np.array([[0.1, 0.2, 0.3], [2.0, 0.0, 0.0]])
    Up = vpm.Vvpm_on_Xs(pf, probes)
    assert Up.shape == (2, 3) and vpm.get_np(pf) == 800
    # The probe velocity equals the field's velocity there (probes carry Γ = 0).
    with Ctx(802) as c:
        c.set(np.vstack([X, probes]), np.vstack([G, np.zeros((2, 3))]),
              np.concatenate([S, [1e-6, 1e-6]]))
        Ur, _ = c.uj(1, L.PREC_FP64, 800, 802)
    assert rel_max(Up, Ur) <= 1e-12
    t0 = pf.t
    vpm.nextstep(pf, 0.005)
    assert abs(pf.t - t0 - 0.005) < 1e-15 and pf.nt == 1
    ens = vpm.monitor_enstrophy(pf)
    cd = vpm.monitor_Cd(pf)
    assert ens > 0 and 0.0 <= cd["cd_zero_ratio"] <= 1.0
    vpm.remove_particle(pf, 799)
    assert vpm.get_np(pf) == 799
    with pytest.raises(ValueError):
        vpm.remove_particle(pf, 3)
    pf.close()


@pytest.mark.parametrize("k", [L.KERNEL_WINCKELMANS, L.KERNEL_GAUSSIANERF])
@pytest.mark.parametrize("nb", [1, 57, 3000])
def test_free_vortex_force_matches_oracle(oracle, k, nb):
    X, G, S = uniform_box(5000, seed_index=130)
    rng = np.random.default_rng(nb)
    Xb = rng.uniform(-1, 1, (nb, 3))
    Gb = rng.normal(0, 1, (nb, 3))
    Sb = rng.uniform(0.05, 0.2, nb)
    Xb[0] = X[10]                      # a bound particle on top of a free one
    M0 = oracle.ffv_direct(k, Xb, Gb, Sb, X, G)
    with Ctx(5000) as c:
        c.set(X, G, S)
        M = np.empty((nb, 6))
        c.rc(c.lib.vpm_ffv_direct(c.p, k, nb, L.dptr(np.ascontiguousarray(Xb)), 3,
                                  L.dptr(np.ascontiguousarray(Gb)), 3,
                                  L.dptr(np.ascontiguousarray(Sb)), 1, L.dptr(M), 6))
    assert rel_l2(M, M0) <= 1e-12 and rel_max(M, M0) <= 1e-11
