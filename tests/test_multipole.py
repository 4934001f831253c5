"""CPU checks of the treecode's far-field arithmetic (the NumPy restatement in
oracle/np_multipole.py of what csrc/tree.cuh computes): the Taylor recurrence
against finite differences, the graded multi-index layout, the cell expansion
against the direct singular Biot-Savart sum, and local expansions about a
target-group centre (M2L, L2P) against the cell expansion."""
import numpy as np
import pytest

from oracle import np_multipole as mp


def test_graded_index_layout_is_a_bijection():
    for q in range(9):
        ks = mp.multi_indices(q)
        assert len(ks) == (q + 1) * (q + 2) * (q + 3) // 6
        assert [mp.midx(*k) for k in ks] == list(range(len(ks)))


def test_taylor_recurrence_matches_finite_differences():
    R = np.array([0.7, -0.4, 0.5])
    b = mp.taylor_coefficients(3, R)
    f = lambda y: 1.0 / np.linalg.norm(R - y)
    h = 1e-3
    e = np.eye(3)
    d1 = (f(h * e[0]) - f(-h * e[0])) / (2 * h)
    d11 = (f(h * e[0]) - 2 * f(0 * e[0]) + f(-h * e[0])) / (h * h) / 2.0
    d12 = (f(h * (e[0] + e[1])) - f(h * (e[0] - e[1])) - f(h * (e[1] - e[0])) + f(-h * (e[0] + e[1]))) / (4 * h * h)
    assert abs(b[mp.midx(1, 0, 0)] - d1) < 1e-6
    assert abs(b[mp.midx(2, 0, 0)] - d11) < 1e-5
    assert abs(b[mp.midx(1, 1, 0)] - d12) < 1e-5


@pytest.mark.parametrize("dist", [0.6, 1.2])
def test_cell_expansion_converges_to_the_direct_sum(dist):
    rng = np.random.default_rng(11)
    Y = rng.uniform(-0.1, 0.1, (300, 3))
    G = rng.normal(0.0, 1.0, (300, 3))
    c = np.zeros(3)
    x = dist * np.array([1.0, 0.3, -0.2])
    U0, J0 = mp.direct_singular(Y, G, x)
    errs = []
    for p in (0, 2, 4, 6):
        U, J = mp.far_field(p, mp.moments(p, Y, G, c), c, x)
        errs.append((np.linalg.norm(U - U0) / np.linalg.norm(U0),
                     np.linalg.norm(J - J0) / np.linalg.norm(J0)))
    for (eu0, ej0), (eu1, ej1) in zip(errs, errs[1:]):
        assert eu1 < 0.3 * eu0 and ej1 < 0.3 * ej0
    assert errs[2][0] < 1e-3 and errs[3][0] < 1e-4
    # J is the gradient of U: trace-free
    U, J = mp.far_field(4, mp.moments(4, Y, G, c), c, x)
    assert abs(np.trace(J)) < 1e-9 * np.abs(J).max()


def test_local_expansion_reproduces_the_cell_expansion():
    # M2L then L2P about a target-group centre equals the cell's own expansion
    # (M2P) at the group's targets up to the local truncation, which falls with
    # the local order q.
    rng = np.random.default_rng(12)
    Y = rng.uniform(-0.1, 0.1, (200, 3))
    G = rng.normal(0.0, 1.0, (200, 3))
    c = np.zeros(3)
    z = np.array([0.9, 0.35, -0.25])
    X = z + rng.uniform(-0.1, 0.1, (20, 3))
    p = 4
    M = mp.moments(p, Y, G, c)
    ref = [mp.far_field(p, M, c, x) for x in X]
    errs = []
    for q in (2, 4, 6, 8):
        L = mp.local_from_moments(p, q, M, c, z)
        got = [mp.local_to_target(q, L, z, x) for x in X]
        eu = max(np.linalg.norm(g[0] - r[0]) / np.linalg.norm(r[0]) for g, r in zip(got, ref))
        ej = max(np.linalg.norm(g[1] - r[1]) / np.linalg.norm(r[1]) for g, r in zip(got, ref))
        errs.append((eu, ej))
    for (eu0, ej0), (eu1, ej1) in zip(errs, errs[1:]):
        assert eu1 < 0.3 * eu0 and ej1 < 0.3 * ej0
    assert errs[2][0] < 1e-4 and errs[2][1] < 1e-3
    # At the group centre the local expansion holds the cell expansion's
    # derivatives exactly (no truncation in ψ, ∂ψ and ∂∂ψ there for q >= 2).
    L = mp.local_from_moments(p, 2, M, c, z)
    U, J = mp.local_to_target(2, L, z, z)
    U0, J0 = mp.far_field(p, M, c, z)
    assert np.allclose(U, U0, rtol=1e-12, atol=0) and np.allclose(J, J0, rtol=1e-10, atol=1e-14)


def _ball(rng, n, r):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1)[:, None]
    return v * (r * rng.random(n) ** (1 / 3))[:, None]


@pytest.mark.parametrize("ratio", [1.0, 1.5, 2.0, 4.0])
def test_local_order_7_matches_m2p_for_cells_not_smaller_than_the_group(ratio):
    # The treecode takes a far cell by the group's local expansion only when the
    # cell's radius R_s is at least the group's R_t.  At the acceptance limit
    # R_t + R_s = θ d (θ = 0.4, the worst case; most far cells lie well inside
    # it), J with local order 7 stays within 1 % of the cell expansion at every
    # target (M2P, p = 4) from R_s = 1.5 R_t on, and within 25 % at equal radii
    # (mean over the trials 5 %), where order 6 is up to twice M2P's error.
    rng = np.random.default_rng(7 + int(10 * ratio))
    theta, p = 0.4, 4
    rt = theta / (1.0 + ratio)
    rs = ratio * rt
    worst = {6: 0.0, 7: 0.0}
    for trial in range(4):
        d = rng.normal(size=3)
        c = d / np.linalg.norm(d)
        Y = c + _ball(rng, 40, rs)
        G = rng.normal(size=(40, 3))
        X = _ball(rng, 12, rt)
        M = mp.moments(p, Y, G, c)
        err = {"m2p": 0.0, 6: 0.0, 7: 0.0}
        ref = 0.0
        Ls = {q: mp.local_from_moments(p, q, M, c, np.zeros(3)) for q in (6, 7)}
        for x in X:
            _, J0 = mp.direct_singular(Y, G, x)
            ref += np.sum(J0 ** 2)
            err["m2p"] += np.sum((mp.far_field(p, M, c, x)[1] - J0) ** 2)
            for q in (6, 7):
                err[q] += np.sum((mp.local_to_target(q, Ls[q], np.zeros(3), x)[1] - J0) ** 2)
        for q in (6, 7):
            worst[q] = max(worst[q], np.sqrt(err[q] / ref) / np.sqrt(err["m2p"] / ref))
    if ratio == 1.0:
        assert worst[7] <= 1.25 and worst[6] > 1.5 * worst[7], worst
    else:
        assert worst[7] <= 1.01, worst
