"""NumPy restatement of the Cartesian multipole far field of the treecode.

TEST INFRASTRUCTURE ONLY: it checks, on the CPU, the expansion arithmetic that
flowunsteady_gb300/csrc/tree.cuh implements on the GPU; the product never
imports it.

FLOWUnsteady's default U/∇U evaluator is `vpm.UJ_fmm` with
`vpm.FMM(p=4, ncrit=50, theta=0.4, nonzero_sigma=false)`
(src/FLOWUnsteady_simulation.jl:38,43): a fast multipole method whose far field
uses the singular kernel.  FLOWExaFMM, which implements it, is not in the
reference tree, so the far-field arithmetic here is restated from the
mathematics:

    ψ(x) = 1/(4π) Σ_j Γ_j / |x - y_j|,   U = ∇ × ψ,   J_ab = ∂U_a/∂x_b,
    1/|x - y| = Σ_k b_k(R) (y - c)^k,    R = x - c,
    b_0 = 1/|R|,  |k| |R|² b_k = (2|k|-1) Σ_i R_i b_{k-e_i} - (|k|-1) Σ_i b_{k-2e_i}

(the Cartesian Taylor recurrence of Lindsay & Krasny 2001), with cell moments
M_k^m = Σ_j Γ_j^m (y_j - c)^k.  The direct singular sum
U = -1/(4π) Σ (x - y) × Γ / |x - y|³ is the check.
"""
from __future__ import annotations

import numpy as np


def multi_indices(q):
    """Multi-indices with |k| <= q in graded order (as midx in tree.cuh)."""
    out = []
    for n in range(q + 1):
        for a in range(n, -1, -1):
            for b in range(n - a, -1, -1):
                out.append((a, b, n - a - b))
    return out


def midx(a, b, c):
    n = a + b + c
    return n * (n + 1) * (n + 2) // 6 + (b + c) * (b + c + 1) // 2 + c


def taylor_coefficients(q, R):
    """b_k(R) for |k| <= q by the recurrence."""
    ks = multi_indices(q)
    R = np.asarray(R, dtype=np.float64)
    r2 = float(R @ R)
    b = np.zeros(len(ks))
    b[0] = 1.0 / np.sqrt(r2)
    for k in ks[1:]:
        n = sum(k)
        s1 = s2 = 0.0
        for i in range(3):
            if k[i] > 0:
                km = list(k); km[i] -= 1
                s1 += R[i] * b[midx(*km)]
            if k[i] > 1:
                km = list(k); km[i] -= 2
                s2 += b[midx(*km)]
        b[midx(*k)] = ((2 * n - 1) * s1 - (n - 1) * s2) / (n * r2)
    return b


def moments(p, Y, G, c):
    """M[m, k] = Σ_j Γ_j^m (y_j - c)^k, |k| <= p."""
    ks = multi_indices(p)
    d = np.asarray(Y, np.float64) - np.asarray(c, np.float64)
    mono = np.stack([np.prod(d ** np.array(k), axis=1) for k in ks], axis=1)   # (nj, NC)
    return np.asarray(G, np.float64).T @ mono                                     # (3, NC)


def far_field(p, M, c, x):
    """U (3,) and J (3, 3) at x from the moments of one cell centred at c."""
    ks = multi_indices(p)
    b = taylor_coefficients(p + 2, np.asarray(x, np.float64) - np.asarray(c, np.float64))
    dpsi = np.zeros((3, 3))          # [i, m] = ∂_i ψ_m
    ddpsi = np.zeros((3, 3, 3))      # [i, j, m]
    for kk, k in enumerate(ks):
        for i in range(3):
            ki = list(k); ki[i] += 1
            dpsi[i] += -(k[i] + 1) * b[midx(*ki)] * M[:, kk]
            for j in range(3):
                kij = list(ki); kij[j] += 1
                ddpsi[i, j] += (k[i] + 1) * (ki[j] + 1) * b[midx(*kij)] * M[:, kk]
    dpsi /= 4 * np.pi
    ddpsi /= 4 * np.pi
    eps = np.zeros((3, 3, 3))
    eps[0, 1, 2] = eps[1, 2, 0] = eps[2, 0, 1] = 1.0
    eps[0, 2, 1] = eps[2, 1, 0] = eps[1, 0, 2] = -1.0
    U = np.einsum("abc,bc->a", eps, dpsi)
    J = np.einsum("acd,bcd->ab", eps, ddpsi)
    return U, J


def direct_singular(Y, G, x):
    """U and J of the singular Biot-Savart law at x from sources Y, G."""
    d = np.asarray(x, np.float64)[None, :] - np.asarray(Y, np.float64)
    r = np.sqrt((d * d).sum(1))
    q = 1.0 / r**3
    qr = -3.0 / r**5
    c = np.cross(d, G)
    U = -(q[:, None] * c).sum(0) / (4 * np.pi)
    eps = np.zeros((3, 3, 3))
    eps[0, 1, 2] = eps[1, 2, 0] = eps[2, 0, 1] = 1.0
    eps[0, 2, 1] = eps[2, 1, 0] = eps[1, 0, 2] = -1.0
    J = np.einsum("j,ja,jb->ab", qr, c, d) + np.einsum("abc,j,jc->ab", eps, q, G)
    return U, -J / (4 * np.pi)


# ---- local expansions (M2L, L2P) ------------------------------------------------
# Not evaluated on the GPU: the treecode evaluates every far cell at every
# target (M2P).  These are the operators of a far field evaluated once per
# target group, checked here first.
# Restated from the same mathematics for a target group centred at z: with
# R = x - c = (z - c) + y and ∂_{R_i} b_k = -(k_i + 1) b_{k+e_i},
#     b_k((z - c) + y) = Σ_j (-1)^{|j|} C(k+j, j) b_{k+j}(z - c) y^j,
# C(k+j, j) = Π_i (k_i + j_i)! / (k_i! j_i!), so the moments of a far cell give
# the local coefficients of ψ (without 1/(4π)) about z,
#     L_j^m = Σ_k M_k^m (-1)^{|j|} C(k+j, j) b_{k+j}(z - c),   |j| <= q,
# and ψ_m(z + y) = Σ_j L_j^m y^j, with ∂ψ and ∂∂ψ from the polynomial.

def _binom_multi(k, j):
    from math import comb
    return comb(k[0] + j[0], j[0]) * comb(k[1] + j[1], j[1]) * comb(k[2] + j[2], j[2])


def local_from_moments(p, q, M, c, z):
    """L[m, j] (3, ncoef(q)) about z from the moments M (3, ncoef(p)) of a cell at c."""
    ks, js = multi_indices(p), multi_indices(q)
    b = taylor_coefficients(p + q, np.asarray(z, np.float64) - np.asarray(c, np.float64))
    L = np.zeros((3, len(js)))
    for jj, j in enumerate(js):
        sgn = -1.0 if sum(j) % 2 else 1.0
        for kk, k in enumerate(ks):
            kj = (k[0] + j[0], k[1] + j[1], k[2] + j[2])
            L[:, jj] += sgn * _binom_multi(k, j) * b[midx(*kj)] * M[:, kk]
    return L


def local_to_target(q, L, z, x):
    """U (3,) and J (3, 3) at x from the local coefficients L about z."""
    js = multi_indices(q)
    y = np.asarray(x, np.float64) - np.asarray(z, np.float64)

    def mono(e):
        return 0.0 if min(e) < 0 else float(np.prod(y ** np.array(e)))

    dpsi = np.zeros((3, 3))          # [i, m] = ∂_i ψ_m
    ddpsi = np.zeros((3, 3, 3))      # [i, l, m]
    for jj, j in enumerate(js):
        for i in range(3):
            if j[i] == 0:
                continue
            ji = list(j); ji[i] -= 1
            dpsi[i] += j[i] * mono(ji) * L[:, jj]
            for l in range(3):
                f = j[i] * (ji[l])
                if f == 0:
                    continue
                jil = list(ji); jil[l] -= 1
                ddpsi[i, l] += f * mono(jil) * L[:, jj]
    dpsi /= 4 * np.pi
    ddpsi /= 4 * np.pi
    eps = np.zeros((3, 3, 3))
    eps[0, 1, 2] = eps[1, 2, 0] = eps[2, 0, 1] = 1.0
    eps[0, 2, 1] = eps[2, 1, 0] = eps[1, 0, 2] = -1.0
    U = np.einsum("abc,bc->a", eps, dpsi)
    J = np.einsum("acd,bcd->ab", eps, ddpsi)
    return U, J
