"""Seeded synthetic particle fields with the shapes of the benchmark workloads.

There is no public dataset for this path; every field is generated from a
NumPy PCG64 generator seeded with 20261203 + workload index.

  uniform_box(n)        N particles uniform in [-1,1]³, Γ ~ N(0, std 1e-3) per
                        component, σ ~ U[0.04, 0.08]          (single U/J evaluation, N=4,096)
  leapfrog_rings()      two coaxial rings R=1, Γ0=1 at z=0 and z=0.8, 200 stations
                        x 19 cross-section particles, σ=0.06  (7,600 particles)
  helical_wake(n)       90% on 3 helices (radius 1, pitch 0.2, 4 turns, phases
                        0/120/240°, N(0,0.01) jitter, Γ tangent, |Γ| = 1/√N_helix),
                        10% uniform in [-1.5,1.5]³ with Γ ~ N(0, 1e-4), σ=0.03
                        (N=262,144; 12 turns for N=1,048,576)
  batch_sizes(48)       48 sizes log-uniform in [2,048, 131,072]
"""
from __future__ import annotations

import numpy as np

SEED0 = 20261203


def rng_for(index: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(SEED0 + index))


def uniform_box(n: int, seed_index: int = 0, gamma_std: float = 1e-3):
    rng = rng_for(seed_index)
    X = rng.uniform(-1.0, 1.0, (n, 3))
    G = rng.normal(0.0, gamma_std, (n, 3))
    S = rng.uniform(0.04, 0.08, n)
    return X, G, S


def leapfrog_rings(nstations: int = 200, R: float = 1.0, Gamma0: float = 1.0,
                   z0: float = 0.0, z1: float = 0.8, sigma: float = 0.06,
                   width: float = 0.05):
    """Two coaxial vortex rings of the same sign.  Each azimuthal station holds a
    centre particle and rings of 6 and 12 particles at radii 0.05 and 0.1 of the
    cross-section; the strengths carry Gaussian cross-section weights
    exp(-r²/(2·width²)) normalised to sum 1, times Γ0·ds along the tangent."""
    layers = [(0.0, 1), (0.05, 6), (0.1, 12)]
    offs, w = [], []
    for rad, cnt in layers:
        for k in range(cnt):
            ang = 2 * np.pi * k / cnt
            offs.append((rad * np.cos(ang), rad * np.sin(ang)))
            w.append(np.exp(-rad**2 / (2 * width**2)))
    w = np.array(w) / np.sum(w)
    ds = 2 * np.pi * R / nstations
    Xs, Gs = [], []
    for zc in (z0, z1):
        for i in range(nstations):
            th = 2 * np.pi * i / nstations
            er = np.array([np.cos(th), np.sin(th), 0.0])
            et = np.array([-np.sin(th), np.cos(th), 0.0])
            ez = np.array([0.0, 0.0, 1.0])
            for (a, b), wk in zip(offs, w):
                Xs.append((R + a) * er + b * ez + np.array([0.0, 0.0, zc]))
                Gs.append(Gamma0 * ds * wk * et)
    X = np.array(Xs)
    G = np.array(Gs)
    S = np.full(X.shape[0], sigma)
    return X, G, S


def helical_wake(n: int, turns: int = 4, seed_index: int = 2, sigma: float = 0.03):
    rng = rng_for(seed_index)
    n_helix_total = int(round(0.9 * n))
    n_each = [n_helix_total // 3] * 3
    n_each[0] += n_helix_total - sum(n_each)
    Xs, Gs = [], []
    pitch = 0.2
    for h, nh in enumerate(n_each):
        phase = 2 * np.pi * h / 3
        t = np.sort(rng.uniform(0.0, 2 * np.pi * turns, nh))
        pos = np.stack([np.cos(t + phase), np.sin(t + phase), pitch * t / (2 * np.pi)], axis=1)
        pos += rng.normal(0.0, 0.01, pos.shape)
        tan = np.stack([-np.sin(t + phase), np.cos(t + phase),
                        np.full_like(t, pitch / (2 * np.pi))], axis=1)
        tan /= np.linalg.norm(tan, axis=1, keepdims=True)
        Xs.append(pos)
        Gs.append(tan / np.sqrt(nh))
    nu = n - n_helix_total
    Xs.append(rng.uniform(-1.5, 1.5, (nu, 3)))
    Gs.append(rng.normal(0.0, 1e-4, (nu, 3)))
    X = np.concatenate(Xs)
    G = np.concatenate(Gs)
    S = np.full(n, sigma)
    return X, G, S


def batch_sizes(nfields: int = 48, lo: int = 2048, hi: int = 131072, seed_index: int = 3):
    rng = rng_for(seed_index)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), nfields)).astype(np.int64)
