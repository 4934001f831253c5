"""The split-source cluster form of the FP32C pair passes.

When a target tile's source range is split into chunks, the chunks either
write their partial sums (FP32C: the (hi, lo) float pairs) into scratch rows
that a second launch sums in fixed order (partial slots), or run as one
thread-block cluster whose CTAs sum each other's compensated (hi, lo) pairs
through distributed shared memory in rank order.  Partial slots are the default (measured faster on GB300);
VPM_CLUSTER=1 takes clusters wherever a cluster size fits.

Checked here, with each form forced in its own process: the cluster form is
taken, matches the CPU FP64 oracle (U/J within 1e-5 relative L2, like every
FP32C pass), agrees with the partial-slot form to FP32 rounding (different
chunk boundaries change the summation order, not the result), is bitwise
repeatable, and carries a dynamic-SFS step as the oracle does."""
import os
import subprocess
import sys

import numpy as np
import pytest

from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300.workloads import uniform_box
from tests.helpers import rel_l2, scheme

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_SCRIPT = r"""
import ctypes, sys, numpy as np
sys.path.insert(0, sys.argv[1])
import torch
from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300.workloads import uniform_box
from tests.helpers import Ctx, scheme
n = int(sys.argv[2])
X, G, S = uniform_box(n, seed_index=170)
S = S * 2.0
out = {}
dev = torch.device("cuda:0")
Xd, Gd, Sd = (torch.tensor(np.ascontiguousarray(a), device=dev) for a in (X.T, G.T, S))
for k in (0, 1):
    for rep in range(2):
        Ud = torch.zeros((3, n), dtype=torch.float64, device=dev)
        Jd = torch.zeros((9, n), dtype=torch.float64, device=dev)
        rc = L.lib().vpm_uj_device_async(k, L.PREC_FP32C, n, Xd.data_ptr(), Gd.data_ptr(),
                                         Sd.data_ptr(), n, n, None, n, Ud.data_ptr(),
                                         Jd.data_ptr(), n, None)
        assert rc == 0, L.last_error()
        torch.cuda.synchronize()
        nc, cl = ctypes.c_int32(), ctypes.c_int32()
        L.lib().vpm_debug_last_plan(None, None, ctypes.byref(nc), ctypes.byref(cl))
        out[f"U{k}{rep}"] = Ud.cpu().numpy().T
        out[f"J{k}{rep}"] = Jd.cpu().numpy().T.reshape(n, 3, 3)
        out[f"plan{k}"] = np.array([nc.value, cl.value])
# An analytic dynamic-SFS step through the context path (every FP32C pass kind).
Xs, Gs, Ss = X[:3000] * 0.5, G[:3000] * 200.0, S[:3000] * 1.5
flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE | L.SFS_ANALYTIC_DSIGMA
with Ctx(3000) as c:
    c.set(Xs, Gs, Ss)
    c.step(scheme(kernel=1, prec=L.PREC_FP32C, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4),
           0.005, nsteps=2)
    out["Xs"], out["Gs"], out["Ss"] = c.state()
np.savez(sys.argv[3], **out)
"""


def run_forced(tmp_path, mode, n):
    out = tmp_path / f"mode{mode}_{n}.npz"
    script = tmp_path / "forced.py"
    script.write_text(_SCRIPT)
    env = dict(os.environ, VPM_CLUSTER=str(mode))
    subprocess.run([sys.executable, str(script), ROOT, str(n), str(out)], check=True, env=env,
                   timeout=600)
    return np.load(out)


@pytest.mark.parametrize("n", [7600, 40000])
def test_cluster_form_against_oracle_and_partial_slots(oracle, tmp_path, n):
    clu = run_forced(tmp_path, 1, n)
    slots = run_forced(tmp_path, 0, n)
    X, G, S = uniform_box(n, seed_index=170)
    S = S * 2.0
    idx = np.random.default_rng(171).choice(n, 600, replace=False)
    for k in (0, 1):
        nc, cl = clu[f"plan{k}"]
        assert nc > 1 and cl == nc                       # the cluster form ran
        nc0, cl0 = slots[f"plan{k}"]
        assert nc0 > 1 and cl0 == 1                      # the partial-slot form ran
        U, J = clu[f"U{k}0"], clu[f"J{k}0"]
        assert np.array_equal(U, clu[f"U{k}1"]) and np.array_equal(J, clu[f"J{k}1"])
        U0, J0 = oracle.uj_direct(k, X, G, S, Xt=X[idx])
        assert rel_l2(U[idx], U0) <= 1e-5 and rel_l2(J[idx], J0) <= 1e-5
        assert rel_l2(U, slots[f"U{k}0"]) <= 1e-6 and rel_l2(J, slots[f"J{k}0"]) <= 1e-6
    # The step: both forms track the oracle on the step increments.
    Xs, Gs, Ss = X[:3000] * 0.5, G[:3000] * 200.0, S[:3000] * 1.5
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE | L.SFS_ANALYTIC_DSIGMA
    sc64 = scheme(kernel=1, prec=L.PREC_FP64, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4)
    Xo, Go, So, _, _ = oracle.step(sc64, Xs, Gs, Ss, None, 0.005, nsteps=2)
    for r in (clu, slots):
        assert rel_l2(r["Xs"] - Xs, Xo - Xs) <= 2e-6
        assert rel_l2(r["Gs"] - Gs, Go - Gs) <= 1e-4
        assert rel_l2(r["Ss"] - Ss, So - Ss) <= 1e-4
