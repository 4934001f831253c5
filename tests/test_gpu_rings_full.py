"""The two-ring leapfrogging run at full length against the CPU FP64 oracle.

The fixtures tests/golden/rings_{analytic,fd}_n7600_400steps.npz hold the
oracle's trajectory of 7,600 particles (Gaussian-erf, transposed rVPM,
dynamic SFS with backscatter clipping and the positive procedure, core
spreading ν = 1e-4, RK3 with dt = 0.005, 400 steps; relaxation off), made by
tests/golden/make_rings_fixture.py: every 50 steps the |Γ|-weighted centroid
and mean radius of each ring, the enstrophy and impulse, the C_d statistics
and the mean σ (src/FLOWUnsteady_monitors.jl:573-574, :614, :697-703 of
FLOWUnsteady), and the final state.

The GPU replays the run with FP64 pair passes (parity: differences at FP64
rounding, amplified by 400 steps of the dynamics) and with FP32C pair passes
(the finite-difference C_d form amplifies FP32 rounding by 1/(1-α) = 1000).
Tolerances are about ten times the differences measured on a GB300."""
import os

import numpy as np
import pytest

from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300.workloads import leapfrog_rings
from tests.helpers import Ctx, rel_l2, scheme

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
I_ENS, I_IZ, I_CDM, I_CDS, I_ZERO, I_SIG = 0, 3, 7, 8, 9, 12

# (form, precision) -> tolerances:
#   rings: max |Δ| of centroids and radii; ens/iz/sig: relative; cdm/cds:
#   relative C_d mean / std; zero: absolute zero ratio; then the final state:
#   dx max |Δx|, g rel-L2 Γ, s max |Δσ|, c rel-L2 C_d.
TOL = {
    ("analytic", L.PREC_FP64): dict(rings=1e-12, ens=1e-12, iz=1e-12, sig=1e-12, cdm=1e-10,
                                    cds=1e-10, zero=3e-4, dx=5e-12, g=2e-12, s=1e-13, c=1e-10),
    ("fd", L.PREC_FP64): dict(rings=2e-11, ens=1e-11, iz=1e-11, sig=1e-12, cdm=1e-9, cds=1e-9,
                              zero=3e-4, dx=5e-10, g=1e-10, s=5e-12, c=1e-9),
    ("analytic", L.PREC_FP32C): dict(rings=1e-5, ens=1e-5, iz=1e-5, sig=5e-4, cdm=1e-3, cds=1e-3,
                                     zero=1e-2, dx=2e-4, g=4e-5, s=1e-2, c=1e-3),
    ("fd", L.PREC_FP32C): dict(rings=1e-3, ens=1e-3, iz=1e-3, sig=3e-3, cdm=0.2, cds=0.3,
                               zero=0.1, dx=1e-2, g=5e-3, s=5e-2, c=0.5),
}


def ring_scheme(form, prec):
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE
    if form == "analytic":
        flags |= L.SFS_ANALYTIC_DSIGMA
    return scheme(kernel=L.KERNEL_GAUSSIANERF, prec=prec, sfs=L.SFS_DYNAMIC, flags=flags,
                  alpha=0.999, rlxf=1.0, minC=0.0, maxC=1.0, nu=1e-4)


def observables(c, n):
    X, G, S = c.state()
    rows = []
    for lo, hi in ((0, n // 2), (n // 2, n)):
        w = np.linalg.norm(G[lo:hi], axis=1)
        cen = (w[:, None] * X[lo:hi]).sum(0) / w.sum()
        rad = (w * np.hypot(X[lo:hi, 0], X[lo:hi, 1])).sum() / w.sum()
        rows.append(np.concatenate([cen, [rad]]))
    return np.concatenate(rows), c.diag(L.KERNEL_GAUSSIANERF, L.PREC_FP64)


def rel(a, b):
    return abs(a - b) / abs(b)


@pytest.mark.parametrize("prec", [L.PREC_FP64, L.PREC_FP32C])
@pytest.mark.parametrize("form", ["analytic", "fd"])
def test_leapfrog_rings_400_steps_track_the_oracle(form, prec):
    d = np.load(os.path.join(GOLD, f"rings_{form}_n7600_400steps.npz"))
    tol = TOL[(form, prec)]
    X, G, S = leapfrog_rings()
    n = X.shape[0]
    sc = ring_scheme(form, prec)
    with Ctx(n) as c:
        c.set(X, G, S)
        for i in range(1, len(d["steps"])):
            c.step(sc, float(d["dt"]), int(d["steps"][i] - d["steps"][i - 1]))
            r, dg = observables(c, n)
            ref_r, ref_d = d["rings"][i], d["diags"][i]
            assert np.abs(r - ref_r).max() <= tol["rings"], (i, r, ref_r)
            assert rel(dg[I_ENS], ref_d[I_ENS]) <= tol["ens"], i
            assert rel(dg[I_IZ], ref_d[I_IZ]) <= tol["iz"], i
            assert rel(dg[I_SIG], ref_d[I_SIG]) <= tol["sig"], i
            assert rel(dg[I_CDM], ref_d[I_CDM]) <= tol["cdm"], i
            assert rel(dg[I_CDS], ref_d[I_CDS]) <= tol["cds"], i
            assert abs(dg[I_ZERO] - ref_d[I_ZERO]) <= tol["zero"], i
        Xg, Gg, Sg = c.state()
        Cg, _ = c.sfs()
    assert np.abs(Xg - d["X"]).max() <= tol["dx"]
    assert rel_l2(Gg, d["G"]) <= tol["g"]
    assert np.abs(Sg - d["S"]).max() <= tol["s"]
    assert rel_l2(Cg[:, 0], d["C"][:, 0]) <= tol["c"]
