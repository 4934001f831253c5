"""GPU parity of the U/∇U pair pass (and the ζ pass behind E_str and the
enstrophy) against the CPU FP64 oracle, through the C ABI.

Tolerances: FP64 pair sums ≤ 1e-12 relative L2 (and ≤ 1e-11 relative max) of
the oracle; FP32C ≤ 1e-5 relative L2 (the target precision)."""
import ctypes
import os

import numpy as np
import pytest

from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300.workloads import helical_wake, uniform_box
from tests.helpers import Ctx, rel_l2, rel_max, scheme

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
KERNELS = [L.KERNEL_WINCKELMANS, L.KERNEL_GAUSSIANERF]


def stretching(J, G):
    return np.einsum("iba,ib->ia", J, G)


@pytest.mark.parametrize("k", KERNELS)
def test_fp64_matches_oracle_uniform_4096(oracle, k):
    X, G, S = uniform_box(4096)
    U0, J0 = oracle.uj_direct(k, X, G, S)
    with Ctx(4096) as c:
        c.set(X, G, S)
        U, J = c.uj(k, L.PREC_FP64)
    assert rel_l2(U, U0) <= 1e-12 and rel_l2(J, J0) <= 1e-12
    assert rel_max(U, U0) <= 1e-11 and rel_max(J, J0) <= 1e-11


@pytest.mark.parametrize("k", KERNELS)
def test_fp32c_within_1e5_of_oracle(oracle, k):
    X, G, S = uniform_box(4096)
    U0, J0 = oracle.uj_direct(k, X, G, S)
    with Ctx(4096) as c:
        c.set(X, G, S)
        U, J = c.uj(k, L.PREC_FP32C)
        Un, Jn = c.uj(k, L.PREC_FP32)
    assert rel_l2(U, U0) <= 1e-5 and rel_l2(J, J0) <= 1e-5
    assert rel_l2(stretching(J, G), stretching(J0, G)) <= 1e-5
    # naive FP32 is reported, not bounded tightly
    assert rel_l2(Un, U0) < 1e-3


@pytest.mark.parametrize("k", KERNELS)
def test_fp32c_helical_wake_sample(oracle, k):
    # 16,384-particle helical wake: dense near field (σ=0.03 with 0.01 jitter).
    X, G, S = helical_wake(16384)
    rng = np.random.default_rng(5)
    idx = np.sort(rng.choice(X.shape[0], 512, replace=False))
    U0, J0 = oracle.uj_direct(k, X, G, S, Xt=X[idx])
    with Ctx(X.shape[0]) as c:
        c.set(X, G, S)
        U, J = c.uj(k, L.PREC_FP32C)
        U64, J64 = c.uj(k, L.PREC_FP64)
    assert rel_l2(U64[idx], U0) <= 1e-12 and rel_l2(J64[idx], J0) <= 1e-12
    assert rel_l2(U[idx], U0) <= 1e-5 and rel_l2(J[idx], J0) <= 1e-5


@pytest.mark.parametrize("name,k", [("winckelmans", 0), ("gaussianerf", 1)])
def test_golden_vectors_on_gpu(name, k):
    d = np.load(os.path.join(GOLD, f"uj_{name}_n160.npz"))
    with Ctx(200) as c:
        c.set(d["X"], d["G"], d["S"])
        U, J = c.uj(k, L.PREC_FP64)
        assert rel_max(U, d["U"]) <= 1e-12 and rel_max(J, d["J"]) <= 1e-12
        U, J = c.uj(k, L.PREC_FP32C)
        assert rel_l2(U, d["U"]) <= 1e-5 and rel_l2(J, d["J"]) <= 1e-5


@pytest.mark.parametrize("n", [1, 2, 3, 31, 33, 257, 1000])
@pytest.mark.parametrize("k", KERNELS)
def test_ragged_sizes(oracle, n, k):
    X, G, S = uniform_box(n, seed_index=40 + n)
    S = S * 4
    U0, J0 = oracle.uj_direct(k, X, G, S)
    with Ctx(n + 5) as c:
        c.set(X, G, S)
        for prec, tol in ((L.PREC_FP64, 1e-12), (L.PREC_FP32C, 1e-5), (L.PREC_FP32, 1e-4)):
            U, J = c.uj(k, prec)
            if n == 1:
                assert np.all(U == 0) and np.all(J == 0)
            else:
                assert rel_l2(U, U0) <= tol and rel_l2(J, J0) <= tol, prec


def test_target_subset_equals_full_rows(oracle):
    # Probe-style evaluation of the tail [2900, 3000) from all 3000 sources.
    X, G, S = uniform_box(3000, seed_index=50)
    U0, J0 = oracle.uj_direct(1, X, G, S, Xt=X[2900:])
    with Ctx(3000) as c:
        c.set(X, G, S)
        U, J = c.uj(1, L.PREC_FP64)
        Us, Js = c.uj(1, L.PREC_FP64, 2900, 3000)
        assert rel_max(Us, U[2900:]) < 1e-13 and rel_max(Js, J[2900:]) < 1e-13
        assert rel_l2(Us, U0) <= 1e-12 and rel_l2(Js, J0) <= 1e-12
        # FP32C: the subset's CTAs use other reference points, so it agrees with
        # the full evaluation to FP32 rounding and with the oracle to 1e-5.
        Us, Js = c.uj(1, L.PREC_FP32C, 2900, 3000)
        assert rel_l2(Us, U0) <= 1e-5 and rel_l2(Js, J0) <= 1e-5


def test_repeatable_bitwise():
    X, G, S = helical_wake(20000)
    with Ctx(20000) as c:
        c.set(X, G, S)
        a = c.uj(1, L.PREC_FP32C)
        b = c.uj(1, L.PREC_FP32C)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_device_pointer_entry_point():
    torch = pytest.importorskip("torch")
    X, G, S = uniform_box(2000, seed_index=60)
    with Ctx(2000) as c:
        c.set(X, G, S)
        U0, J0 = c.uj(0, L.PREC_FP32C)
    dev = torch.device("cuda:0")
    Xd = torch.tensor(X.T.copy(), device=dev)
    Gd = torch.tensor(G.T.copy(), device=dev)
    Sd = torch.tensor(S, device=dev)
    Ud = torch.zeros((3, 2000), dtype=torch.float64, device=dev)
    Jd = torch.zeros((9, 2000), dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream().cuda_stream
    rc = L.lib().vpm_uj_device_async(0, L.PREC_FP32C, 2000, Xd.data_ptr(), Gd.data_ptr(),
                                     Sd.data_ptr(), 2000, 2000, None, 2000, Ud.data_ptr(),
                                     Jd.data_ptr(), 2000, ctypes.c_void_p(st))
    assert rc == 0, L.last_error()
    torch.cuda.synchronize()
    U = Ud.cpu().numpy().T
    J = Jd.cpu().numpy().T.reshape(2000, 3, 3)
    assert rel_max(U, U0) < 1e-12 and rel_max(J, J0) < 1e-12


@pytest.mark.parametrize("k", KERNELS)
def test_estr_and_enstrophy_match_oracle(oracle, k):
    X, G, S = uniform_box(1500, seed_index=70)
    S = S * 3
    U0, J0 = oracle.uj_direct(k, X, G, S)
    E0, om0 = oracle.estr_direct(k, X, G, S, J0, transposed=True)
    d0 = oracle.diagnostics(k, X, G, S)
    sc = scheme(kernel=k, prec=L.PREC_FP64, sfs=L.SFS_CONSTANT, flags=0)
    with Ctx(1500) as c:
        c.set(X, G, S)
        c.rc(c.lib.vpm_eval_sfs(c.p, ctypes.byref(sc)))
        _, E = c.sfs()
        assert rel_l2(E, E0) <= 1e-11
        d = c.diag(k, L.PREC_FP64)
        assert abs(d[0] - d0[0]) <= 1e-12 * abs(d0[0])
        assert np.allclose(d[1:7], d0[1:7], rtol=1e-12, atol=1e-18)
        sc.precision = L.PREC_FP32C
        c.rc(c.lib.vpm_eval_sfs(c.p, ctypes.byref(sc)))
        _, E = c.sfs()
        assert rel_l2(E, E0) <= 1e-5
        d = c.diag(k, L.PREC_FP32C)
        assert abs(d[0] - d0[0]) <= 1e-6 * abs(d0[0])


_PLAIN_STAGING_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
from tests.helpers import Ctx
from flowunsteady_gb300.workloads import helical_wake
import ctypes
from flowunsteady_gb300 import _lib as L
X, G, S = helical_wake(int(sys.argv[2]))
out = {}
with Ctx(X.shape[0]) as c:
    c.set(X, G, S)
    for k in (0, 1):
        for p in (1, 2):
            c.rc(c.lib.vpm_set_tile(c.p, k, p, ctypes.byref(L.Tile(128, 2, 0, 0))))
    for k in (0, 1):
        for p in (1, 2):
            out[f"U{k}{p}"], out[f"J{k}{p}"] = c.uj(k, p)
    out["Us"], out["Js"] = c.uj(1, 2, 1000, 1777)
np.savez(sys.argv[3], **out)
"""


@pytest.mark.parametrize("n", [20001, 4096])
def test_bulk_copy_staging_matches_plain_loads_bitwise(tmp_path, n):
    # The U/J FP32 passes stage source tiles with cp.async.bulk; VPM_NO_TMA=1
    # forces plain loads.  Same conversion and summation order: identical bits.
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = tmp_path / "plain.npz"
    script = tmp_path / "plain.py"
    script.write_text(_PLAIN_STAGING_SCRIPT)
    env = dict(os.environ, VPM_NO_TMA="1")
    subprocess.run([sys.executable, str(script), root, str(n), str(out)], check=True, env=env,
                   timeout=300)
    ref = np.load(out)
    X, G, S = helical_wake(n)
    with Ctx(n) as c:
        c.set(X, G, S)
        for k in (0, 1):       # same tile shape in both processes
            for p in (1, 2):
                c.rc(c.lib.vpm_set_tile(c.p, k, p, ctypes.byref(L.Tile(128, 2, 0, 0))))
        for k in (0, 1):
            for p in (1, 2):
                U, J = c.uj(k, p)
                assert np.array_equal(U, ref[f"U{k}{p}"]) and np.array_equal(J, ref[f"J{k}{p}"])
        Us, Js = c.uj(1, 2, 1000, 1777)
        assert np.array_equal(Us, ref["Us"]) and np.array_equal(Js, ref["Js"])


@pytest.mark.parametrize("n", [3001, 40000])
def test_context_and_device_pointer_paths_agree_bitwise(n):
    # The context path (TMA staging) and the device-pointer entry point (plain
    # loads) plan the same launch and sum the source-chunk partials in the same
    # slot order: identical bits.
    torch = pytest.importorskip("torch")
    X, G, S = uniform_box(n, seed_index=70 + n % 7)
    with Ctx(n) as c:
        c.set(X, G, S)
        U0, J0 = c.uj(1, L.PREC_FP32C)
        U1, J1 = c.uj(0, L.PREC_FP64)
    dev = torch.device("cuda:0")
    Xd, Gd, Sd = (torch.tensor(a, device=dev) for a in (X.T.copy(), G.T.copy(), S))
    for k, p, U_ref, J_ref in ((1, L.PREC_FP32C, U0, J0), (0, L.PREC_FP64, U1, J1)):
        Ud = torch.zeros((3, n), dtype=torch.float64, device=dev)
        Jd = torch.zeros((9, n), dtype=torch.float64, device=dev)
        rc = L.lib().vpm_uj_device_async(k, p, n, Xd.data_ptr(), Gd.data_ptr(), Sd.data_ptr(), n,
                                         n, None, n, Ud.data_ptr(), Jd.data_ptr(), n, None)
        assert rc == 0
        torch.cuda.synchronize()
        assert np.array_equal(Ud.cpu().numpy().T, U_ref)
        assert np.array_equal(Jd.cpu().numpy().T.reshape(n, 3, 3), J_ref)


_GENERAL_FORMS_SCRIPT = r"""
import sys, ctypes, numpy as np
sys.path.insert(0, sys.argv[1])
from tests.helpers import Ctx, scheme
from flowunsteady_gb300.workloads import helical_wake
from flowunsteady_gb300 import _lib as L
X, G, S = helical_wake(int(sys.argv[2]))
flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE | L.SFS_ANALYTIC_DSIGMA
out = {}
with Ctx(X.shape[0]) as c:
    c.set(X, G, S)
    for p in (1, 2):
        c.rc(c.lib.vpm_set_tile(c.p, 1, p, ctypes.byref(L.Tile(128, 2, 0, 0))))
    for p in (1, 2):
        out[f"U{p}"], out[f"J{p}"] = c.uj(1, p)
    sc = scheme(kernel=1, prec=L.PREC_FP32C, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4)
    c.rc(c.lib.vpm_eval_sfs(c.p, ctypes.byref(sc)))
    out["C"], out["E"] = c.sfs()
    c.step(sc, 1e-4, nsteps=2)
    out["X"], out["G"], out["S"] = c.state()
np.savez(sys.argv[3], **out)
"""


def test_gaussian_far_field_forms_match_general_forms(tmp_path, oracle):
    # Warp/32-source blocks with ρ² >= 50 at every pair take q = 1/r³,
    # p = -3/r⁵, and blocks where ζ underflows to zero are skipped in the ζ
    # passes; VPM_NO_FARFIELD=1 forces the general forms everywhere.  The
    # helical wake (coherent particle order) takes the far forms for most blocks.
    import subprocess
    import sys
    n = 30000
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = tmp_path / "general.npz"
    script = tmp_path / "general.py"
    script.write_text(_GENERAL_FORMS_SCRIPT)
    env = dict(os.environ, VPM_NO_FARFIELD="1")
    subprocess.run([sys.executable, str(script), root, str(n), str(out)], check=True, env=env,
                   timeout=300)
    ref = np.load(out)
    X, G, S = helical_wake(n)
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE | L.SFS_ANALYTIC_DSIGMA
    with Ctx(n) as c:
        c.set(X, G, S)
        for p in (1, 2):
            c.rc(c.lib.vpm_set_tile(c.p, 1, p, ctypes.byref(L.Tile(128, 2, 0, 0))))
        for p in (1, 2):
            U, J = c.uj(1, p)
            # The far forms agree with the general ones to FP32 rounding; the
            # compensated sums fold at other points (after general blocks).
            assert rel_l2(U, ref[f"U{p}"]) <= 5e-7 and rel_l2(J, ref[f"J{p}"]) <= 5e-7
        sc = scheme(kernel=1, prec=L.PREC_FP32C, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4)
        c.rc(c.lib.vpm_eval_sfs(c.p, ctypes.byref(sc)))
        C, E = c.sfs()
        # E = S(J_p, Ω_p) - Σ ζ S(J_q, Γ_q) nearly cancels: a few hundred times
        # the relative difference of J.
        assert rel_l2(E, ref["E"]) <= 1e-4 and rel_l2(C, ref["C"]) <= 1e-3
        c.step(sc, 1e-4, nsteps=2)
        Xs, Gs, Ss = c.state()
    assert np.abs(Xs - ref["X"]).max() <= 1e-7 and rel_l2(Gs, ref["G"]) <= 5e-6
    assert rel_max(Ss, ref["S"]) <= 1e-7
    # And both against the FP64 oracle on a target sample.
    idx = np.sort(np.random.default_rng(9).choice(n, 400, replace=False))
    U0, J0 = oracle.uj_direct(1, X, G, S, Xt=X[idx])
    assert rel_l2(ref["U2"][idx], U0) <= 1e-5 and rel_l2(ref["J2"][idx], J0) <= 1e-5


def test_morton_ordered_passes_match_original_order(oracle):
    # Fields of 65,536 particles or more are evaluated along a Morton curve
    # (vpm_set_particle_order(VPM_ORDER_CALLER) turns it off): only the
    # summation order changes.  The particle order here is random, the case
    # the curve is for.
    n = 70000
    X, G, S = helical_wake(n)
    order = np.random.default_rng(5).permutation(n)
    X, G, S = X[order], G[order], S[order]
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE | L.SFS_ANALYTIC_DSIGMA
    sc = scheme(kernel=1, prec=L.PREC_FP32C, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4)
    out = {}
    for mode in (L.ORDER_CALLER, L.ORDER_AUTO):
        with Ctx(n) as c:
            c.rc(c.lib.vpm_set_particle_order(c.p, mode))
            c.set(X, G, S)
            if mode == L.ORDER_CALLER:   # the FP64 reference, in the caller's order
                out["U64"], out["J64"] = c.uj(1, L.PREC_FP64)
                sc64 = scheme(kernel=1, prec=L.PREC_FP64, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4)
                c.rc(c.lib.vpm_eval_sfs(c.p, ctypes.byref(sc64)))
                out["C64"], out["E64"] = c.sfs()
            r = out.setdefault(mode, {})
            r["U"], r["J"] = c.uj(1, L.PREC_FP32C)
            c.rc(c.lib.vpm_eval_sfs(c.p, ctypes.byref(sc)))
            r["C"], r["E"] = c.sfs()
            c.step(sc, 1e-4, nsteps=2)
            r["X"], r["G"], r["S"] = c.state()
    srt, ref = out[L.ORDER_AUTO], out[L.ORDER_CALLER]
    err = {}
    for tag, r in (("", srt), ("_unsorted", ref)):
        err["U" + tag] = rel_l2(r["U"], out["U64"])
        err["J" + tag] = rel_l2(r["J"], out["J64"])
        err["E" + tag] = rel_l2(r["E"], out["E64"])
        err["C" + tag] = rel_l2(r["C"][:, 0], out["C64"][:, 0])
    err["X_steps"] = float(np.abs(srt["X"] - ref["X"]).max())
    err["G_steps"] = rel_l2(srt["G"], ref["G"])
    err["S_steps"] = rel_l2(srt["S"], ref["S"])
    assert err["U"] <= 5e-7 and err["J"] <= 5e-7, err
    assert err["U_unsorted"] <= 1e-5 and err["J_unsorted"] <= 1e-5, err
    # E = S(J_p, Ω_p) - Σ ζ S(J_q, Γ_q) nearly cancels: its FP32 error is a few
    # hundred times that of J (7e-5 for coherent particle orders).
    assert err["E"] <= 2e-4 and err["E_unsorted"] <= 2e-4, err
    assert err["C"] <= 2e-3 and err["C_unsorted"] <= 2e-3, err
    # Two steps of dt = 1e-4 carry the U differences (|U| ~ 500) into x.
    assert err["X_steps"] <= 1e-7 and err["G_steps"] <= 5e-6 and err["S_steps"] <= 1e-8, err
    idx = np.sort(np.random.default_rng(6).choice(n, 300, replace=False))
    U0, J0 = oracle.uj_direct(1, X, G, S, Xt=X[idx])
    assert rel_l2(srt["U"][idx], U0) <= 1e-5 and rel_l2(srt["J"][idx], J0) <= 1e-5


def test_jacobian_row_order_is_dU_a_dx_b():
    # The C ABI's J is row-major per particle: J[3a+b] = dU_a/dx_b.  Pin it
    # through the ABI against central differences of U at zero-strength probes
    # (probes carry Γ = 0, so they change nothing): the orientation that
    # FLOWVPM's classic stretching S = J·Γ and its transposed form rely on.
    X, G, S = uniform_box(600, seed_index=61)
    S = S * 3.0
    rng = np.random.default_rng(62)
    pts = rng.uniform(-0.6, 0.6, (5, 3))
    h = 1e-5
    probes = [pts]
    for b in range(3):
        e = np.zeros(3)
        e[b] = h
        probes += [pts + e, pts - e]
    P = np.vstack(probes)
    m = P.shape[0]
    with Ctx(600 + m) as c:
        c.set(X, G, S)
        c.append(P, np.zeros_like(P), np.full(m, 1e-6))
        U, J = c.uj(L.KERNEL_GAUSSIANERF, L.PREC_FP64, 600, 600 + m)
    Jc = J[:5]
    fd = np.empty((5, 3, 3))
    for b in range(3):
        up, um = U[5 + 10 * b:10 + 10 * b], U[10 + 10 * b:15 + 10 * b]
        fd[:, :, b] = (up - um) / (2 * h)       # column b: dU_a/dx_b for a = 0..2
    assert rel_l2(Jc, fd) <= 1e-7
    assert rel_l2(np.transpose(Jc, (0, 2, 1)), fd) > 1e-2


@pytest.mark.parametrize("chunk", [1, 128, 300, 1000, 100000])
def test_pinned_source_chunk_matches_oracle(oracle, chunk):
    # vpm_set_tile's chunk pins the source range of a work item (rounded up to
    # whole tiles of the block size); every split goes through the partial
    # slots and their fixed-order reduction.  A negative length is refused.
    from flowunsteady_gb300.workloads import leapfrog_rings
    X, G, S = leapfrog_rings()
    n = X.shape[0]
    idx = np.sort(np.random.default_rng(31).choice(n, 300, replace=False))
    U0, J0 = oracle.uj_direct(L.KERNEL_GAUSSIANERF, X, G, S, Xt=X[idx])
    with Ctx(n) as c:
        c.set(X, G, S)
        Ud, Jd = c.uj(L.KERNEL_GAUSSIANERF, L.PREC_FP32C)
        t = L.Tile(128, 2, chunk, 0)
        c.rc(c.lib.vpm_set_tile(c.p, L.KERNEL_GAUSSIANERF, L.PREC_FP32C, ctypes.byref(t)))
        U, J = c.uj(L.KERNEL_GAUSSIANERF, L.PREC_FP32C)
        bad = L.Tile(128, 2, -1, 0)
        assert c.lib.vpm_set_tile(c.p, L.KERNEL_GAUSSIANERF, L.PREC_FP32C, ctypes.byref(bad)) == L.ERR_INVALID
    assert rel_l2(U[idx], U0) <= 1e-5 and rel_l2(J[idx], J0) <= 1e-5
    assert rel_l2(U, Ud) <= 1e-6 and rel_l2(J, Jd) <= 1e-6
