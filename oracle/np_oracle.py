"""Independent NumPy restatement of the rVPM pair sums, for small N.

TEST INFRASTRUCTURE ONLY (a second, independently written checker of the C++
oracle in vpm_oracle.cpp; the product never imports it).  PARITY UNPINNED, for
the reason given in oracle/oracle.py.

It is written from the kernel functions g(ρ), g'(ρ), ζ(ρ) rather than from the
closed forms the C++ oracle uses:
    q(r)      = g(r/σ) / r³
    (dq/dr)/r = (ρ g'(ρ) - 3 g(ρ)) / r⁵
    U         = -1/(4π) Σ q (Δx × Γ)                         rvpm.md:88-99
    J_ab      = -1/(4π) Σ [(dq/dr)/r (Δx×Γ)_a Δx_b + q ε_abc Γ_c]
    E_str     = Σ ζ_σq (Γ_q·∇)(u_p - u_q)                     rvpm.md:251-262
(paths inside byuflowlab/FLOWUnsteady).  It evaluates all pairs at once
(O(N²) memory), so keep N below a few thousand.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

WINCKELMANS = 0
GAUSSIANERF = 1

_EPS = np.zeros((3, 3, 3))
_EPS[0, 1, 2] = _EPS[1, 2, 0] = _EPS[2, 0, 1] = 1.0
_EPS[0, 2, 1] = _EPS[2, 1, 0] = _EPS[1, 0, 2] = -1.0


def g_dg(kernel, rho):
    rho = np.asarray(rho, dtype=np.float64)
    if kernel == WINCKELMANS:
        s = rho**2 + 1.0
        return rho**3 * (rho**2 + 2.5) / s**2.5, 7.5 * rho**2 / s**3.5
    e = np.exp(-0.5 * rho**2)
    c = np.sqrt(2.0 / np.pi)
    return erf(rho / np.sqrt(2.0)) - c * rho * e, c * rho**2 * e


def zeta(kernel, rho):
    rho = np.asarray(rho, dtype=np.float64)
    if kernel == WINCKELMANS:
        return 15.0 / (8.0 * np.pi) * (rho**2 + 1.0) ** -3.5
    return np.exp(-0.5 * rho**2) / (2.0 * np.pi) ** 1.5


def uj(kernel, X, G, S, Xt=None, sigma_scale=1.0):
    X = np.asarray(X, np.float64)
    G = np.asarray(G, np.float64)
    S = np.asarray(S, np.float64) * sigma_scale
    Xt = X if Xt is None else np.asarray(Xt, np.float64)
    d = Xt[:, None, :] - X[None, :, :]                # (nt, ns, 3)
    r = np.sqrt(np.einsum("ijk,ijk->ij", d, d))
    mask = r > 0
    rs = np.where(mask, r, 1.0)
    rho = rs / S[None, :]
    g, dg = g_dg(kernel, rho)
    q = np.where(mask, g / rs**3, 0.0)
    qr = np.where(mask, (rho * dg - 3.0 * g) / rs**5, 0.0)
    c = np.cross(d, G[None, :, :])                    # Δx × Γ
    U = -np.einsum("ij,ijk->ik", q, c) / (4 * np.pi)
    J = np.einsum("ij,ija,ijb->iab", qr, c, d)
    J += np.einsum("abc,ij,jc->iab", _EPS, q, G)
    return U, -J / (4 * np.pi)


def stretch(J, v, transposed=True):
    return np.einsum("iba,ib->ia", J, v) if transposed else np.einsum("iab,ib->ia", J, v)


def estr(kernel, X, G, S, J, transposed=True, sigma_scale=1.0):
    """E_str (n,3) from the pair form Σ_q ζ (J_p - J_q)⋆Γ_q, and ω (n,3) incl. self."""
    X = np.asarray(X, np.float64)
    G = np.asarray(G, np.float64)
    S = np.asarray(S, np.float64) * sigma_scale
    d = X[:, None, :] - X[None, :, :]
    r = np.sqrt(np.einsum("ijk,ijk->ij", d, d))
    z = zeta(kernel, r / S[None, :]) / S[None, :] ** 3      # includes the self term
    om = np.einsum("pq,qk->pk", z, G)
    zx = np.where(r > 0, z, 0.0)
    E = None
    if J is not None:
        dJ = J[:, None, :, :] - J[None, :, :, :]             # (p, q, 3, 3)
        if transposed:
            s = np.einsum("pqba,qb->pqa", dJ, G)
        else:
            s = np.einsum("pqab,qb->pqa", dJ, G)
        E = np.einsum("pq,pqa->pa", zx, s)
    return E, om


def step_rk3(kernel, X, G, S, dt, f=0.0, g=0.2, transposed=True, uinf=(0, 0, 0), nu=0.0):
    """One low-storage RK3 step (Williamson 1980) of the rVPM ODEs without SFS."""
    X, G, S = (np.array(a, np.float64) for a in (X, G, S))
    A = (0.0, -5.0 / 9.0, -153.0 / 128.0)
    B = (1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0)
    qx = np.zeros_like(X)
    qg = np.zeros_like(G)
    qs = np.zeros_like(S)
    qs2 = np.zeros_like(S)
    for a, b in zip(A, B):
        U, J = uj(kernel, X, G, S)
        Sv = stretch(J, G, transposed)
        gg = np.einsum("ik,ik->i", G, G)
        Z = (f + g) / (1 + 3 * f) * np.einsum("ik,ik->i", Sv, G) / gg
        qx = a * qx + dt * (U + np.asarray(uinf))
        qg = a * qg + dt * (Sv - 3.0 * Z[:, None] * G)
        qs = a * qs - dt * S * Z
        X = X + b * qx
        G = G + b * qg
        S = S + b * qs
        if nu > 0:
            qs2 = a * qs2 + dt * 2 * nu
            S = np.sqrt(S**2 + b * qs2)
    return X, G, S


def ffv(kernel, Xb, Gb, Sb, Xf, Gf):
    """Free-vortex force terms (nb, 6), written from the two cross products of
    _Ffv_direct (src/FLOWUnsteady_processing_force.jl:900-921)."""
    d = Xf[None, :, :] - Xb[:, None, :]                        # (nb, nf, 3) = x_f - x_b
    r = np.sqrt(np.einsum("bfk,bfk->bf", d, d))
    mask = r > 0
    rs = np.where(mask, r, 1.0)
    g, _ = g_dg(kernel, rs / Sb[:, None])
    k = np.where(mask, g / (4 * np.pi * rs**3), 0.0)
    U = -k[:, :, None] * np.cross(d, np.broadcast_to(Gb[:, None, :], d.shape))
    M1 = np.einsum("bfk->bk", np.cross(U, np.broadcast_to(Gf[None, :, :], d.shape)))
    gxg = np.cross(np.broadcast_to(Gb[:, None, :], d.shape), np.broadcast_to(Gf[None, :, :], d.shape))
    M2 = np.einsum("bf,bfk->bk", k, np.cross(d, gxg))
    return np.concatenate([M1, M2], axis=1)
