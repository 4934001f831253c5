"""GPU time steps under every scheme switch of vpm_scheme against the CPU FP64
oracle, through the C ABI:

  - classic stretching S = J·Γ (vpm_transposed = false,
    src/FLOWUnsteady_simulation.jl:41,132 of FLOWUnsteady);
  - classic VPM, f = g = 0 (docs/src/theory/rvpm.md:237);
  - rVPM with f != 0 and the dynamic SFS model, which brings in the
    f/(1+3f) E_str terms of dΓ/dt and dσ/dt (rvpm.md:196-236), with the
    finite-difference and the analytic σ-derivative;
  - the SFS model with a prescribed C_d (no dynamic procedure);
  - classic stretching with the dynamic SFS model (E_str then uses J·Γ too).

Each case runs two RK3 steps.  FP64 pair passes: positions and core sizes
within 1e-12 relative (max), strengths within 1e-9 relative (max), C_d within
1e-7.  FP32C pair passes, measured on the increments of the two steps
(x - x0, Γ - Γ0, σ - σ0) in relative L2: positions within 2e-6, strengths and
core sizes within 2e-5 (measured: 2-3e-7 and up to 1.8e-6).  Where the
finite-difference C_d enters, its 1/(1-α) = 1000 amplification of FP32
rounding moves C_d by ~1e-3 relative: positions within 1e-3, strengths and
core sizes within 1e-2 (measured: up to 7e-5 and 8e-4)."""
import numpy as np
import pytest

from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300.workloads import uniform_box
from tests.helpers import Ctx, rel_l2, rel_max, scheme

pytestmark = pytest.mark.gpu

DYN = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE
ANA = DYN | L.SFS_ANALYTIC_DSIGMA

# name -> (scheme keywords, whether the finite-difference C_d is involved)
CASES = {
    "classic": (dict(transposed=0), False),
    "cvpm": (dict(f=0.0, g=0.0), False),
    "rvpm_f_dynamic_fd": (dict(f=0.3, g=0.2, sfs=L.SFS_DYNAMIC, flags=DYN, rlxf=0.5), True),
    "rvpm_f_dynamic_analytic": (dict(f=0.3, g=0.2, sfs=L.SFS_DYNAMIC, flags=ANA, rlxf=0.5), False),
    "constant_cd": (dict(sfs=L.SFS_CONSTANT, Cd=0.13, flags=L.SFS_CLIP_BACKSCATTER), False),
    "constant_cd_f": (dict(f=0.5, g=0.1, sfs=L.SFS_CONSTANT, Cd=0.13, flags=0), False),
    "classic_dynamic_analytic": (dict(transposed=0, sfs=L.SFS_DYNAMIC, flags=ANA), False),
    "cvpm_euler": (dict(f=0.0, g=0.0, integration=L.INTEGRATION_EULER), False),
}


def field(n=320, seed=140):
    X, G, S = uniform_box(n, seed_index=seed)
    return X * 0.5, G * 200.0, S * 3.0


def run_case(oracle, kernel, prec, kw):
    X, G, S = field()
    nu = 1e-4 if kernel == L.KERNEL_GAUSSIANERF else 0.0
    sc = scheme(kernel=kernel, prec=prec, nu=nu, uinf=(0.05, 0.0, -0.02), **kw)
    sc64 = scheme(kernel=kernel, prec=L.PREC_FP64, nu=nu, uinf=(0.05, 0.0, -0.02), **kw)
    Xo, Go, So, Co, Eo = oracle.step(sc64, X, G, S, None, 0.01, nsteps=2)
    with Ctx(X.shape[0]) as c:
        c.set(X, G, S)
        c.step(sc, 0.01, nsteps=2)
        Xg, Gg, Sg = c.state()
        Cg, Eg = c.sfs()
    return (Xg, Gg, Sg, Cg, Eg), (Xo, Go, So, Co, Eo)


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("kernel", [L.KERNEL_WINCKELMANS, L.KERNEL_GAUSSIANERF])
def test_scheme_fp64_matches_oracle(oracle, name, kernel):
    kw, _ = CASES[name]
    (Xg, Gg, Sg, Cg, Eg), (Xo, Go, So, Co, Eo) = run_case(oracle, kernel, L.PREC_FP64, kw)
    assert rel_max(Xg, Xo) <= 1e-12
    assert rel_max(Gg, Go) <= 1e-9
    assert rel_max(Sg, So) <= 1e-12
    if kw.get("sfs", L.SFS_NONE) != L.SFS_NONE:
        assert rel_max(Cg[:, 0], Co[:, 0]) <= 1e-7
        assert rel_max(Eg, Eo) <= 1e-9
        if kw["sfs"] == L.SFS_CONSTANT:
            # Free particles carry the prescribed C_d unless backscatter clipping zeroed it.
            cd = Cg[:, 0]
            assert np.all((cd == 0.13) | ((cd == 0.0) & bool(kw["flags"] & L.SFS_CLIP_BACKSCATTER)))
            assert np.any(cd == 0.13)


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("kernel", [L.KERNEL_WINCKELMANS, L.KERNEL_GAUSSIANERF])
def test_scheme_fp32c_tracks_oracle(oracle, name, kernel):
    kw, fd = CASES[name]
    X0, G0, S0 = field()
    (Xg, Gg, Sg, _, _), (Xo, Go, So, _, _) = run_case(oracle, kernel, L.PREC_FP32C, kw)
    assert rel_l2(Xg - X0, Xo - X0) <= (1e-3 if fd else 2e-6)
    assert rel_l2(Gg - G0, Go - G0) <= (1e-2 if fd else 2e-5)
    assert rel_l2(Sg - S0, So - S0) <= (1e-2 if fd else 2e-5)


def test_classic_and_transposed_differ():
    # The switch reaches the update: the two stretching forms give different Γ.
    X, G, S = field(200, 141)
    out = []
    for tr in (0, 1):
        with Ctx(200) as c:
            c.set(X, G, S)
            c.step(scheme(kernel=1, prec=L.PREC_FP64, transposed=tr), 0.01)
            out.append(c.state()[1])
    assert rel_l2(out[0], out[1]) > 1e-6
