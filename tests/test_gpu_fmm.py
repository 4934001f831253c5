"""GPU treecode (vpm_eval_UJ_fmm, the role of FLOWVPM's UJ_fmm): against the
FP64 oracle's direct sum, its convergence in θ and p, the near-field limit
where it must reproduce the direct FP32C sum, and the far field by local
expansions (M2L, L2P) against the same oracle and against M2P."""
import ctypes

import numpy as np
import pytest

from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300.workloads import helical_wake, uniform_box
from tests.helpers import Ctx, rel_l2

pytestmark = pytest.mark.gpu


def fmm(p=4, ncrit=50, theta=0.4, sigma_factor=7.1, local_order=0):
    f = L.Fmm()
    f.p, f.ncrit, f.theta, f.sigma_factor = p, ncrit, theta, sigma_factor
    f.local_order = local_order
    return f


def eval_fmm(c, k, prec, f):
    c.rc(c.lib.vpm_eval_UJ_fmm(c.p, k, prec, ctypes.byref(f)))
    n = c.np()
    U, J = np.empty((n, 3)), np.empty((n, 3, 3))
    c.rc(c.lib.vpm_get_UJ(c.p, 0, n, L.dptr(U), 3, L.dptr(J), 9))
    return U, J


def stats(c):
    out = (ctypes.c_int64 * len(L.FMM_STATS))()
    c.rc(c.lib.vpm_fmm_stats(c.p, out))
    d = dict(zip(L.FMM_STATS, out))
    return d["cells"], d["leaves"], d["far_entries"], d["near_entries"]


def all_stats(c):
    out = (ctypes.c_int64 * len(L.FMM_STATS))()
    c.rc(c.lib.vpm_fmm_stats(c.p, out))
    return dict(zip(L.FMM_STATS, out))


def test_defaults_follow_flowunsteady():
    f = L.default_fmm()
    assert (f.p, f.ncrit, f.theta) == (4, 50, 0.4) and f.sigma_factor == 7.1
    assert f.local_order == 7


@pytest.mark.parametrize("k", [L.KERNEL_WINCKELMANS, L.KERNEL_GAUSSIANERF])
def test_local_expansions_match_oracle_and_m2p(oracle, k):
    # Far cells at least as large as the target group by one local expansion of
    # order 7 per group: as accurate against the oracle's direct sum as M2P at
    # every target (within 10 %), with fewer (target, cell) moment evaluations.
    n = 60000
    X, G, S = helical_wake(n)
    idx = np.sort(np.random.default_rng(4).choice(n, 600, replace=False))
    U0, J0 = oracle.uj_direct(k, X, G, S, Xt=X[idx])
    with Ctx(n) as c:
        c.set(X, G, S)
        Up, Jp = eval_fmm(c, k, L.PREC_FP32C, fmm(local_order=0))
        sp = all_stats(c)
        Ul, Jl = eval_fmm(c, k, L.PREC_FP32C, fmm(local_order=7))
        sl = all_stats(c)
    assert sp["local_terms"] == 0 and sl["local_terms"] > 0
    assert sl["far_entries"] == sp["far_entries"]
    assert sl["far_evaluations"] < sp["far_evaluations"]
    epu, epj = rel_l2(Up[idx], U0), rel_l2(Jp[idx], J0)
    elu, elj = rel_l2(Ul[idx], U0), rel_l2(Jl[idx], J0)
    assert elu <= 1.1 * epu + 1e-7 and elj <= 1.1 * epj + 1e-7, (epu, epj, elu, elj)
    assert elu <= 1e-4 and elj <= 1e-4
    # The two far forms differ by the local truncation only.
    assert rel_l2(Ul, Up) <= 1e-4 and rel_l2(Jl, Jp) <= 1e-4


def test_local_expansions_leave_fp64_and_other_orders_on_m2p():
    # FP64 and p != 4 take M2P throughout: the results are those of local_order 0.
    X, G, S = helical_wake(12000)
    with Ctx(12000) as c:
        c.set(X, G, S)
        for prec, p in ((L.PREC_FP64, 4), (L.PREC_FP32C, 2)):
            U0, J0 = eval_fmm(c, 1, prec, fmm(p=p, local_order=0))
            U1, J1 = eval_fmm(c, 1, prec, fmm(p=p, local_order=7))
            assert all_stats(c)["local_terms"] == 0
            assert np.array_equal(U0, U1) and np.array_equal(J0, J1)
        bad = fmm(local_order=6)
        assert c.lib.vpm_eval_UJ_fmm(c.p, 1, L.PREC_FP32C, ctypes.byref(bad)) == L.ERR_UNSUPPORTED


@pytest.mark.parametrize("k", [L.KERNEL_WINCKELMANS, L.KERNEL_GAUSSIANERF])
def test_treecode_matches_direct_sum_helical_wake(oracle, k):
    X, G, S = helical_wake(40000)
    idx = np.sort(np.random.default_rng(3).choice(40000, 500, replace=False))
    U0, J0 = oracle.uj_direct(k, X, G, S, Xt=X[idx])
    with Ctx(40000) as c:
        c.set(X, G, S)
        U, J = eval_fmm(c, k, L.PREC_FP32C, fmm())
        cells, leaves, nfar, nnear = stats(c)
        assert leaves > 40000 // 50 and cells > leaves and nfar > 0 and nnear > 0
        eu, ej = rel_l2(U[idx], U0), rel_l2(J[idx], J0)
        assert eu <= 1e-4 and ej <= 1e-4, (eu, ej)
        # Tighter settings converge to the direct sum.  Winckelmans cores
        # differ from the singular far-field kernel by 1.875 (σ/r)^4, so far
        # cells also have to be further away in core sizes.
        tight = fmm(p=6, theta=0.25, sigma_factor=30.0 if k == L.KERNEL_WINCKELMANS else 7.1)
        U6, J6 = eval_fmm(c, k, L.PREC_FP32C, tight)
        e6u, e6j = rel_l2(U6[idx], U0), rel_l2(J6[idx], J0)
        assert e6u <= 0.2 * eu + 2e-6 and e6j <= 0.2 * ej + 2e-6, (eu, ej, e6u, e6j)


def test_near_field_limit_equals_direct_fp32c():
    # With every cell too close to be far, the treecode is the direct sum.
    X, G, S = uniform_box(6000, seed_index=140)
    with Ctx(6000) as c:
        c.set(X, G, S)
        Ud, Jd = c.uj(1, L.PREC_FP32C)
        U, J = eval_fmm(c, 1, L.PREC_FP32C, fmm(theta=0.01))
        assert stats(c)[2] == 0
    assert rel_l2(U, Ud) <= 1e-6 and rel_l2(J, Jd) <= 1e-6


def test_fp64_treecode_converges_with_order(oracle):
    X, G, S = helical_wake(12000)
    U0, J0 = oracle.uj_direct(1, X, G, S)
    errs = []
    with Ctx(12000) as c:
        c.set(X, G, S)
        for p in (2, 4, 6):
            U, J = eval_fmm(c, 1, L.PREC_FP64, fmm(p=p, theta=0.4))
            errs.append((rel_l2(U, U0), rel_l2(J, J0)))
        # near-field limit in FP64: the oracle to FP64 rounding
        U, J = eval_fmm(c, 1, L.PREC_FP64, fmm(theta=0.01))
        assert rel_l2(U, U0) <= 1e-12 and rel_l2(J, J0) <= 1e-12
    assert errs[1][0] < errs[0][0] and errs[2][0] < errs[1][0]
    assert errs[2][0] < 1e-5


def test_coincident_and_tiny_fields():
    X, G, S = uniform_box(300, seed_index=141)
    X[299] = X[0]
    with Ctx(400) as c:
        c.set(X[:1], G[:1], S[:1])
        U, J = eval_fmm(c, 1, L.PREC_FP32C, fmm())
        assert np.all(U == 0) and np.all(J == 0)
        c.set(X, G, S)
        Ud, Jd = c.uj(1, L.PREC_FP32C)
        U, J = eval_fmm(c, 1, L.PREC_FP32C, fmm(ncrit=8))
        assert np.all(np.isfinite(U)) and np.all(np.isfinite(J))
        assert rel_l2(U, Ud) <= 1e-3 and rel_l2(J, Jd) <= 1e-2
        bad = fmm(p=3)
        assert c.lib.vpm_eval_UJ_fmm(c.p, 1, L.PREC_FP32C, ctypes.byref(bad)) == L.ERR_UNSUPPORTED


@pytest.mark.parametrize("sfs", [False, True])
def test_step_with_treecode_tracks_direct_step(sfs):
    # vpm_step with uj_method = VPM_UJ_TREE: the plain U/J passes by the
    # treecode (the α-derivative and ζ passes of the dynamic SFS stay direct).
    from tests.helpers import scheme
    X, G, S = helical_wake(20000)
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE | L.SFS_ANALYTIC_DSIGMA
    kw = dict(kernel=1, prec=L.PREC_FP32C, nu=1e-4)
    if sfs:
        kw.update(sfs=L.SFS_DYNAMIC, flags=flags)
    sd = scheme(**kw)
    st = scheme(**kw)
    st.uj_method = L.UJ_TREE
    st.fmm = L.default_fmm()
    with Ctx(20000) as a, Ctx(20000) as b:
        a.set(X, G, S)
        b.set(X, G, S)
        a.step(sd, 1e-4, nsteps=3)
        b.step(st, 1e-4, nsteps=3)
        Xa, Ga, Sa = a.state()
        Xb, Gb, Sb = b.state()
    assert np.all(np.isfinite(Xb)) and np.all(np.isfinite(Gb))
    assert np.abs(Xb - Xa).max() <= 1e-6
    assert rel_l2(Gb, Ga) <= 1e-4 and rel_l2(Sb, Sa) <= 1e-6


@pytest.mark.parametrize("analytic", [True, False])
def test_sfs_passes_from_treecode_match_direct(analytic):
    # With uj_method = VPM_UJ_TREE and Gaussian-erf FP32, the analytic SFS
    # passes (U/J + DJ, ζ + Dζ) run over the tree's near lists; the
    # finite-difference form keeps its σ and ασ passes on the direct sum.
    from tests.helpers import scheme
    X, G, S = helical_wake(20000)
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE
    if analytic:
        flags |= L.SFS_ANALYTIC_DSIGMA
    sd = scheme(kernel=1, prec=L.PREC_FP32C, sfs=L.SFS_DYNAMIC, flags=flags)
    st = scheme(kernel=1, prec=L.PREC_FP32C, sfs=L.SFS_DYNAMIC, flags=flags)
    st.uj_method = L.UJ_TREE
    st.fmm = L.default_fmm()
    with Ctx(20000) as c:
        c.set(X, G, S)
        c.rc(c.lib.vpm_eval_sfs(c.p, ctypes.byref(sd)))
        C0, E0 = c.sfs()
        U0, J0 = np.empty((20000, 3)), np.empty((20000, 3, 3))
        c.rc(c.lib.vpm_get_UJ(c.p, 0, 20000, L.dptr(U0), 3, L.dptr(J0), 9))
        c.set(X, G, S)
        c.rc(c.lib.vpm_eval_sfs(c.p, ctypes.byref(st)))
        C1, E1 = c.sfs()
        U1, J1 = np.empty((20000, 3)), np.empty((20000, 3, 3))
        c.rc(c.lib.vpm_get_UJ(c.p, 0, 20000, L.dptr(U1), 3, L.dptr(J1), 9))
    assert rel_l2(U1, U0) <= 1e-4 and rel_l2(J1, J0) <= 1e-4
    assert rel_l2(E1, E0) <= 1e-3, rel_l2(E1, E0)
    assert rel_l2(C1[:, 0], C0[:, 0]) <= (1e-2 if analytic else 1e-12), rel_l2(C1[:, 0], C0[:, 0])
