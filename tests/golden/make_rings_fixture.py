"""Generate the full-length leapfrogging-ring fixtures from the CPU FP64 oracle.

The workload is the two-ring rVPM run: 2 x 200 stations x 19 cross-section
particles = 7,600 particles, Gaussian-erf kernel, transposed rVPM (f = 0,
g = 1/5), dynamic SFS (pseudo-three-level, positive, backscatter clipping),
core spreading with nu = 1e-4, low-storage RK3 with dt = 0.005, 400 steps,
relaxation off.  Scheme defaults follow src/FLOWUnsteady_simulation.jl:127-137
of FLOWUnsteady; the monitored quantities follow src/FLOWUnsteady_monitors.jl
(enstrophy :573-574 and :614, C_d statistics :697-703).

FLOWVPM is not available here, so the trajectory is the oracle's
(oracle/vpm_oracle.cpp), not the reference's: the fixture pins the GPU path
against the oracle over the whole run.  Two fixtures are written, one per form
of the dynamic procedure's sigma-derivative (finite difference between the
sigma and alpha*sigma filter levels; analytic d/d(alpha)).  Each holds, every
50 steps, the |Gamma|-weighted centroid and mean radius of each ring, the
impulse, the enstrophy and the C_d statistics, plus the final state.

Run from the repository root (about 17 minutes per form on 8 cores):
    python tests/golden/make_rings_fixture.py [fd|analytic]...
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from flowunsteady_gb300 import _lib as L  # noqa: E402
from flowunsteady_gb300.workloads import leapfrog_rings  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
NSTEPS = 400
EVERY = 50
DT = 0.005


def ring_scheme(analytic):
    """The two-ring run's scheme: Gaussian-erf, FP64, RK3, transposed rVPM,
    dynamic SFS with backscatter clipping and the positive procedure, nu = 1e-4."""
    s = L.default_scheme()
    s.kernel, s.precision = L.KERNEL_GAUSSIANERF, L.PREC_FP64
    s.sfs = L.SFS_DYNAMIC
    s.sfs_flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE
    if analytic:
        s.sfs_flags |= L.SFS_ANALYTIC_DSIGMA
    s.sfs_alpha, s.sfs_rlxf, s.sfs_minC, s.sfs_maxC = 0.999, 1.0, 0.0, 1.0
    s.nu = 1e-4
    return s


def observables(X, G, S, C, nhalf):
    """Per ring: |Γ|-weighted centroid (3) and mean radius; then the oracle's
    diagnostics vector (enstrophy, impulse, ΣΓ, C_d statistics, mean σ)."""
    rows = []
    for lo, hi in ((0, nhalf), (nhalf, 2 * nhalf)):
        w = np.linalg.norm(G[lo:hi], axis=1)
        c = (w[:, None] * X[lo:hi]).sum(0) / w.sum()
        rad = (w * np.hypot(X[lo:hi, 0], X[lo:hi, 1])).sum() / w.sum()
        rows.append(np.concatenate([c, [rad]]))
    d = O.diagnostics(L.KERNEL_GAUSSIANERF, X, G, S, C)
    return np.concatenate(rows), d


def run(form):
    analytic = form == "analytic"
    X, G, S = leapfrog_rings()
    n = X.shape[0]
    C = np.zeros((n, 3))
    sc = ring_scheme(analytic)
    steps, rings, diags = [], [], []
    r, d = observables(X, G, S, C, n // 2)
    steps.append(0); rings.append(r); diags.append(d)
    t0 = time.perf_counter()
    for s0 in range(0, NSTEPS, EVERY):
        X, G, S, C, _ = O.step(sc, X, G, S, C, DT, nsteps=EVERY)
        r, d = observables(X, G, S, C, n // 2)
        steps.append(s0 + EVERY); rings.append(r); diags.append(d)
        print(f"{form}: step {s0 + EVERY}/{NSTEPS}  {time.perf_counter() - t0:.0f} s", flush=True)
    path = os.path.join(OUT, f"rings_{form}_n7600_400steps.npz")
    np.savez_compressed(path, steps=np.array(steps), rings=np.array(rings),
                        diags=np.array(diags), X=X, G=G, S=S, C=C, dt=DT,
                        nsteps=NSTEPS, threads=O.max_threads())
    print("wrote", path)


if __name__ == "__main__":
    forms = sys.argv[1:] or ["analytic", "fd"]
    for f in forms:
        if f not in ("fd", "analytic"):
            raise SystemExit(f"unknown form {f!r}: fd or analytic")
        run(f)
