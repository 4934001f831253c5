"""Generate the golden vectors under tests/golden/ from the CPU FP64 oracle.

FLOWVPM (the Julia package holding the reference arithmetic) is not vendored
with FLOWUnsteady and Julia is absent, so these fixtures are outputs of the
oracle restatement (oracle/vpm_oracle.cpp), cross-checked at generation time
against the independent NumPy restatement (oracle/np_oracle.py).  They pin the
oracle against silent change and give the GPU tests fixed expected values.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from oracle import np_oracle as P  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def field(n, seed, smin=0.04, smax=0.08):
    rng = np.random.Generator(np.random.PCG64(seed))
    X = rng.uniform(-1, 1, (n, 3))
    G = rng.normal(0, 1e-3, (n, 3))
    S = rng.uniform(smin, smax, n)
    return X, G, S


def main():
    for kname, k in (("winckelmans", O.WINCKELMANS), ("gaussianerf", O.GAUSSIANERF)):
        # Wide cores so that near pairs (small ρ) are well represented.
        X, G, S = field(160, 20261203 + 10 + k, 0.1, 0.4)
        U, J = O.uj_direct(k, X, G, S)
        U2, J2 = P.uj(k, X, G, S)
        assert np.abs(U - U2).max() <= 1e-12 * np.abs(U2).max()
        assert np.abs(J - J2).max() <= 1e-12 * np.abs(J2).max()
        E, om = O.estr_direct(k, X, G, S, J, transposed=True)
        E2, om2 = P.estr(k, X, G, S, J, transposed=True)
        assert np.abs(E - E2).max() <= 1e-11 * np.abs(E2).max()
        assert np.abs(om - om2).max() <= 1e-12 * np.abs(om2).max()
        np.savez_compressed(os.path.join(OUT, f"uj_{kname}_n160.npz"), X=X, G=G, S=S, U=U, J=J,
                            E=E, omega=om)
    # One RK3 step of rVPM without SFS (checked against the NumPy RK3).
    X, G, S = field(96, 20261203 + 20, 0.1, 0.3)
    G *= 100.0
    sc = _scheme(kernel=O.GAUSSIANERF, sfs=0, nu=0.0)
    Xn, Gn, Sn, _, _ = O.step(sc, X, G, S, None, dt=0.01)
    Xp, Gp, Sp = P.step_rk3(O.GAUSSIANERF, X, G, S, 0.01)
    assert np.abs(Xn - Xp).max() < 1e-12 and np.abs(Gn - Gp).max() < 1e-12 * np.abs(Gp).max()
    assert np.abs(Sn - Sp).max() < 1e-13
    np.savez_compressed(os.path.join(OUT, "step_rk3_gaussianerf_n96.npz"), X=X, G=G, S=S, Xn=Xn,
                        Gn=Gn, Sn=Sn, dt=0.01)
    print("golden vectors written to", OUT)


def _scheme(**kw):
    from flowunsteady_gb300._lib import Scheme
    s = Scheme()
    s.kernel = kw.get("kernel", 1)
    s.precision = 0
    s.integration = 1
    s.transposed = 1
    s.f, s.g = 0.0, 0.2
    s.nu = kw.get("nu", 0.0)
    s.sfs = kw.get("sfs", 0)
    s.sfs_flags = 1
    s.sfs_alpha, s.sfs_rlxf, s.sfs_minC, s.sfs_maxC = 0.999, 1.0, 0.0, 1.0
    return s


if __name__ == "__main__":
    main()
