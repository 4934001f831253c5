"""The fused reduction of split source ranges.

When a target tile's sources are split into chunks, every chunk writes its
partial sums into its slot (FP64 values, or the FP32 passes' float pairs).
Either a second launch sums the slots in chunk order, or (the fused form) the
last CTA of each tile to finish sums them, in the same order and arithmetic,
inside the pair launch.  The planner fuses the passes of large
fields; VPM_FUSED_REDUCE=1 fuses every split pass and =0 none.

Checked here, with each form forced in its own process: the fused form runs
(one launch fewer per split pass), gives bitwise the values of the separate
reduction for U/J (FP32C and FP64), a target subset, the two stateless entry
points (the no-alloc one with its static scratch), and three dynamic-SFS RK3
steps, and matches the CPU FP64 oracle."""
import os
import subprocess
import sys

import numpy as np
import pytest

from flowunsteady_gb300.workloads import uniform_box
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_SCRIPT = r"""
import ctypes, sys, numpy as np
sys.path.insert(0, sys.argv[1])
from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300.workloads import uniform_box
from tests.helpers import Ctx, scheme
n = int(sys.argv[2])
X, G, S = uniform_box(n, seed_index=180)
S = S * 2.0
out = {}
with Ctx(n) as c:
    c.set(X, G, S)
    for k in (0, 1):
        for p in (L.PREC_FP32C, L.PREC_FP64):
            l0 = ctypes.c_int64()
            c.rc(L.lib().vpm_get_launch_count(c.p, ctypes.byref(l0)))
            out[f"U{k}{p}"], out[f"J{k}{p}"] = c.uj(k, p)
            l1 = ctypes.c_int64()
            c.rc(L.lib().vpm_get_launch_count(c.p, ctypes.byref(l1)))
            out[f"launches{k}{p}"] = np.array(l1.value - l0.value)
    out["Us"], out["Js"] = c.uj(1, L.PREC_FP32C, 1000, n - 777)
# The stateless entry points (caller's device arrays; the no-alloc one keeps
# the slots and the tile counters in its static scratch): all targets, and
# 3,000 probe targets against all sources.
import torch
dev = torch.device("cuda:0")
Xd, Gd, Sd = (torch.tensor(np.ascontiguousarray(a), device=dev) for a in (X.T, G.T, S))
Xp = torch.tensor(np.ascontiguousarray(X[:3000].T * 0.9), device=dev)
for name in ("vpm_uj_device_async", "vpm_uj_device_noalloc"):
    fn = getattr(L.lib(), name)
    for m, Xt in ((n, None), (3000, Xp)):
        if name.endswith("noalloc") and m > 16384:
            continue
        Ud = torch.zeros((3, m), dtype=torch.float64, device=dev)
        Jd = torch.zeros((9, m), dtype=torch.float64, device=dev)
        rc = fn(1, L.PREC_FP32C, n, Xd.data_ptr(), Gd.data_ptr(), Sd.data_ptr(), n, m,
                None if Xt is None else Xt.data_ptr(), m, Ud.data_ptr(), Jd.data_ptr(), m, None)
        assert rc == 0, L.last_error()
        torch.cuda.synchronize()
        out[f"{name}_{m}_U"] = Ud.cpu().numpy().T
        out[f"{name}_{m}_J"] = Jd.cpu().numpy().T
flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE | L.SFS_ANALYTIC_DSIGMA
with Ctx(n) as c:
    c.set(X * 0.5, G * 200.0, S * 1.5)
    c.rc(L.lib().vpm_step(c.p, 0.005, ctypes.byref(scheme(kernel=1, prec=L.PREC_FP32C,
         sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4)), 3, 0))
    out["Xs"], out["Gs"], out["Ss"] = c.state()
np.savez(sys.argv[3], **out)
"""


def run_forced(tmp_path, mode, n):
    out = tmp_path / f"fused{mode}_{n}.npz"
    script = tmp_path / "forced.py"
    script.write_text(_SCRIPT)
    env = dict(os.environ, VPM_FUSED_REDUCE=str(mode))
    subprocess.run([sys.executable, str(script), ROOT, str(n), str(out)], check=True, env=env,
                   timeout=600)
    return np.load(out)


@pytest.mark.parametrize("n", [7600, 40000])
def test_fused_reduction_is_bitwise_the_separate_one(oracle, tmp_path, n):
    fused = run_forced(tmp_path, 1, n)
    sep = run_forced(tmp_path, 0, n)
    for key in sep.files:
        if key.startswith("launches"):
            # FP32C U/J splits the sources at both sizes: one launch fewer.
            if key.endswith("2"):
                assert fused[key] == sep[key] - 1, key
            continue
        assert np.array_equal(fused[key], sep[key]), key
    X, G, S = uniform_box(n, seed_index=180)
    S = S * 2.0
    idx = np.random.default_rng(181).choice(n, 500, replace=False)
    for k in (0, 1):
        U0, J0 = oracle.uj_direct(k, X, G, S, Xt=X[idx])
        assert rel_l2(fused[f"U{k}2"][idx], U0) <= 1e-5
        assert rel_l2(fused[f"J{k}2"][idx], J0) <= 1e-5
        assert rel_l2(fused[f"U{k}0"][idx], U0) <= 1e-12
        assert rel_l2(fused[f"J{k}0"][idx], J0) <= 1e-12
