"""CPU checks of the FP64 oracle (no GPU): known answers, an independent NumPy
restatement, invariants and the committed golden vectors."""
import os

import numpy as np
import pytest

from oracle import np_oracle as P
from tests.helpers import rel_max, scheme

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def field(n, seed, smin=0.04, smax=0.08):
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.uniform(-1, 1, (n, 3)), rng.normal(0, 1e-3, (n, 3)), rng.uniform(smin, smax, n)


@pytest.mark.parametrize("k", [0, 1])
def test_oracle_matches_numpy(oracle, k):
    X, G, S = field(200, 1 + k, 0.05, 0.4)
    U, J = oracle.uj_direct(k, X, G, S)
    U2, J2 = P.uj(k, X, G, S)
    assert rel_max(U, U2) < 1e-13 and rel_max(J, J2) < 1e-13
    for tr in (0, 1):
        E, om = oracle.estr_direct(k, X, G, S, J, transposed=tr)
        E2, om2 = P.estr(k, X, G, S, J, transposed=tr)
        assert rel_max(E, E2) < 1e-12 and rel_max(om, om2) < 1e-13


@pytest.mark.parametrize("k", [0, 1])
def test_gradient_is_derivative_of_velocity(oracle, k):
    X, G, S = field(120, 7 + k, 0.1, 0.3)
    Xs, Gs, Ss, Xt = X[6:], G[6:], S[6:], X[:6]
    _, J = oracle.uj_direct(k, Xs, Gs, Ss, Xt=Xt)
    h = 1e-5
    for b in range(3):
        e = np.zeros(3)
        e[b] = h
        Up, _ = oracle.uj_direct(k, Xs, Gs, Ss, Xt=Xt + e)
        Um, _ = oracle.uj_direct(k, Xs, Gs, Ss, Xt=Xt - e)
        assert rel_max((Up - Um) / (2 * h), J[:, :, b]) < 1e-7


@pytest.mark.parametrize("k", [0, 1])
def test_velocity_divergence_free(oracle, k):
    X, G, S = field(300, 11 + k)
    _, J = oracle.uj_direct(k, X, G, S)
    tr = np.trace(J, axis1=1, axis2=2)
    assert np.abs(tr).max() < 1e-12 * np.abs(J).max()


def test_pair_antisymmetry_equal_cores(oracle):
    # Two particles with equal σ and equal Γ: induced velocities are opposite.
    X = np.array([[0.0, 0.0, 0.0], [0.3, -0.1, 0.2]])
    G = np.array([[0.1, 0.2, -0.3], [0.1, 0.2, -0.3]])
    S = np.array([0.2, 0.2])
    for k in (0, 1):
        U, _ = oracle.uj_direct(k, X, G, S)
        assert np.allclose(U[0], -U[1], rtol=1e-14, atol=0)


def test_kernel_known_answers(oracle):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    rho = np.array([1e-4, 1e-2, 0.1, 0.3, 0.49, 0.51, 1.0, 2.0, 5.0])
    g, dg, z = oracle.kernel_eval(1, rho)
    for r, gv, dgv, zv in zip(rho, g, dg, z):
        r = mp.mpf(float(r))
        ge = mp.erf(r / mp.sqrt(2)) - mp.sqrt(2 / mp.pi) * r * mp.e ** (-r**2 / 2)
        assert abs(gv - float(ge)) <= 1e-14 * abs(float(ge))
        assert abs(dgv - float(mp.sqrt(2 / mp.pi) * r**2 * mp.e ** (-r**2 / 2))) <= 1e-14 * abs(dgv)
        assert abs(zv - float(mp.e ** (-r**2 / 2) / (2 * mp.pi) ** 1.5)) <= 1e-14 * zv
    g, dg, z = oracle.kernel_eval(0, rho)
    for r, gv, dgv, zv in zip(rho, g, dg, z):
        r = mp.mpf(float(r))
        assert abs(gv - float(r**3 * (r**2 + 2.5) / (r**2 + 1) ** 2.5)) <= 1e-14 * gv
        assert abs(dgv - float(7.5 * r**2 / (r**2 + 1) ** 3.5)) <= 1e-14 * dgv
        assert abs(zv - float(15 / (8 * mp.pi) / (r**2 + 1) ** 3.5)) <= 1e-14 * zv


def test_kernel_consistency_g_prime_is_4pi_r2_zeta(oracle):
    rho = np.linspace(0.01, 6, 50)
    for k in (0, 1):
        g, dg, z = oracle.kernel_eval(k, rho)
        assert np.allclose(dg, 4 * np.pi * rho**2 * z, rtol=1e-13)
        # g(ρ) = ∫ g' dρ
        fine = np.linspace(0, 6, 200001)
        gf, dgf, _ = oracle.kernel_eval(k, fine)
        integ = np.concatenate([[0], np.cumsum((dgf[1:] + dgf[:-1]) / 2 * np.diff(fine))])
        assert np.allclose(np.interp(rho, fine, integ), g, atol=1e-8)


@pytest.mark.parametrize("name,k", [("winckelmans", 0), ("gaussianerf", 1)])
def test_golden_vectors(oracle, name, k):
    d = np.load(os.path.join(GOLD, f"uj_{name}_n160.npz"))
    U, J = oracle.uj_direct(k, d["X"], d["G"], d["S"])
    assert rel_max(U, d["U"]) < 1e-14 and rel_max(J, d["J"]) < 1e-14
    E, om = oracle.estr_direct(k, d["X"], d["G"], d["S"], J)
    assert rel_max(E, d["E"]) < 1e-13 and rel_max(om, d["omega"]) < 1e-14


def test_golden_rk3_step(oracle):
    d = np.load(os.path.join(GOLD, "step_rk3_gaussianerf_n96.npz"))
    Xn, Gn, Sn, _, _ = oracle.step(scheme(kernel=1), d["X"], d["G"], d["S"], None, float(d["dt"]))
    assert np.abs(Xn - d["Xn"]).max() < 1e-14
    assert rel_max(Gn, d["Gn"]) < 1e-13 and np.abs(Sn - d["Sn"]).max() < 1e-15


def test_rk3_matches_numpy_with_core_spreading(oracle):
    X, G, S = field(64, 31, 0.1, 0.3)
    G *= 50
    Xn, Gn, Sn, _, _ = oracle.step(scheme(kernel=1, nu=1e-3), X, G, S, None, 0.02)
    Xp, Gp, Sp = P.step_rk3(1, X, G, S, 0.02, nu=1e-3)
    assert np.abs(Xn - Xp).max() < 1e-13 and rel_max(Gn, Gp) < 1e-12
    assert np.abs(Sn - Sp).max() < 1e-14


def test_core_spreading_exact_for_constant_rate(oracle):
    # d(σ²)/dt = 2ν is integrated exactly by the RK3 weights: with Γ ⟂ stretching
    # removed (single particle), σ² grows by 2ν·dt per step.
    X = np.zeros((1, 3))
    G = np.array([[0.0, 0.0, 1e-3]])
    S = np.array([0.06])
    _, _, Sn, _, _ = oracle.step(scheme(kernel=1, nu=1e-4), X, G, S, None, 0.005, nsteps=10)
    assert abs(Sn[0] ** 2 - (0.06**2 + 2e-4 * 0.05)) < 1e-15


def test_impulse_conserved_inviscid(oracle):
    # Hydrodynamic impulse ½Σ x×Γ of an isolated ring is conserved by the rVPM
    # equations up to time-discretisation error.
    from flowunsteady_gb300.workloads import leapfrog_rings
    X, G, S = leapfrog_rings(nstations=40, sigma=0.2)
    X, G, S = X[: X.shape[0] // 2], G[: G.shape[0] // 2], S[: S.shape[0] // 2]
    d0 = oracle.diagnostics(1, X, G, S)
    Xn, Gn, Sn, _, _ = oracle.step(scheme(kernel=1), X, G, S, None, 0.01, nsteps=5)
    d1 = oracle.diagnostics(1, Xn, Gn, Sn)
    assert abs(d1[3] - d0[3]) < 1e-4 * abs(d0[3])


def test_thin_ring_self_induced_speed(oracle):
    # Coarse sanity check: a ring of radius R with a Gaussian core of standard
    # deviation s translates at about Γ/(4πR)(ln(8R/δ) - 0.558), δ = √2 s
    # (Saffman's result for a Gaussian core).  The discrete ring has s ≈
    # √(σ² + w²) with particle core σ = 0.06 and cross-section width w = 0.05.
    from flowunsteady_gb300.workloads import leapfrog_rings
    X, G, S = leapfrog_rings(nstations=200, sigma=0.06)
    half = X.shape[0] // 2
    U, _ = oracle.uj_direct(1, X[:half], G[:half], S[:half])
    uz = np.mean(U[:, 2])
    delta = np.sqrt(2.0) * np.hypot(0.06, 0.05)
    saffman = 1.0 / (4 * np.pi) * (np.log(8 / delta) - 0.558)
    assert 0.85 * saffman < uz < 1.15 * saffman


@pytest.mark.parametrize("k", [0, 1])
def test_analytic_sigma_derivatives_match_finite_differences(oracle, k):
    # d/dα at α = 1 of J(ασ) and E_str(ασ) against central differences in α.
    X, G, S = field(150, 41 + k, 0.08, 0.3)
    DJ = oracle.uj_dsigma(k, X, G, S)
    h = 1e-5
    _, Jp = oracle.uj_direct(k, X, G, S, sigma_scale=1 + h)
    _, Jm = oracle.uj_direct(k, X, G, S, sigma_scale=1 - h)
    assert rel_max(DJ, (Jp - Jm) / (2 * h)) < 1e-7
    _, J = oracle.uj_direct(k, X, G, S)
    for tr in (0, 1):
        DE = oracle.estr_dsigma(k, X, G, S, J, DJ, transposed=tr)
        Ep, _ = oracle.estr_direct(k, X, G, S, Jp, transposed=tr, sigma_scale=1 + h)
        Em, _ = oracle.estr_direct(k, X, G, S, Jm, transposed=tr, sigma_scale=1 - h)
        assert rel_max(DE, (Ep - Em) / (2 * h)) < 1e-6


def test_analytic_and_finite_difference_dynamic_cd_agree(oracle):
    # Both dynamic procedures estimate the same C_d up to O(1 - α).
    X, G, S = field(200, 45, 0.1, 0.3)
    X *= 0.5
    G *= 300
    fd = scheme(kernel=1, sfs=1, flags=1 | 2)
    an = scheme(kernel=1, sfs=1, flags=1 | 2 | 4)
    _, _, _, Cf, _ = oracle.step(fd, X, G, S, None, 0.005)
    _, _, _, Ca, _ = oracle.step(an, X, G, S, None, 0.005)
    m = (Cf[:, 0] != 0) & (Ca[:, 0] != 0)
    assert m.sum() > 20
    assert np.median(np.abs(Ca[m, 0] - Cf[m, 0]) / np.abs(Cf[m, 0])) < 1e-2


@pytest.mark.parametrize("k", [0, 1])
def test_free_vortex_force_matches_numpy(oracle, k):
    rng = np.random.default_rng(60 + k)
    Xb, Gb, Sb = rng.uniform(-1, 1, (40, 3)), rng.normal(0, 1, (40, 3)), rng.uniform(0.1, 0.3, 40)
    Xf, Gf = rng.uniform(-1, 1, (300, 3)), rng.normal(0, 1e-2, (300, 3))
    Xf[7] = Xb[3]   # coincident pair: skipped
    M = oracle.ffv_direct(k, Xb, Gb, Sb, Xf, Gf)
    M2 = P.ffv(k, Xb, Gb, Sb, Xf, Gf)
    assert rel_max(M, M2) < 1e-12


def test_cd_statistics_follow_monitor_cd(oracle):
    # vpm.monitor_Cd's record (src/FLOWUnsteady_monitors.jl:697-703): over the
    # free particles with C_d != 0, mean, std, skewness, excess kurtosis,
    # min, max; the zero ratio over all free particles.
    from flowunsteady_gb300.workloads import uniform_box
    X, G, S = uniform_box(500, seed_index=30)
    rng = np.random.default_rng(31)
    C = np.zeros((500, 3))
    C[:, 0] = np.where(rng.random(500) < 0.3, 0.0, rng.normal(0.1, 0.05, 500))
    d = oracle.diagnostics(1, X, G, S * 3, C, n_static=20)
    c = C[:480, 0]
    nz = c[c != 0]
    m = nz.mean()
    m2, m3, m4 = (((nz - m) ** k).mean() for k in (2, 3, 4))
    assert abs(d[7] - m) <= 1e-14 and abs(d[8] - np.sqrt(m2)) <= 1e-14
    assert abs(d[14] - m3 / m2**1.5) <= 1e-12 and abs(d[15] - (m4 / m2**2 - 3)) <= 1e-12
    assert d[9] == (c == 0).mean() and d[10] == nz.min() and d[11] == nz.max()
