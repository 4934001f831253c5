"""Drivers of the reference workloads (seeded synthetic inputs), each printing one JSON result.

    python -m flowunsteady_gb300.runs sweep     # precision sweep, N = 262,144 helical wake
    python -m flowunsteady_gb300.runs rings     # two leapfrogging rings, full rVPM, 400 RK3 steps
    python -m flowunsteady_gb300.runs batch     # 48 fields, log-uniform N in [2,048, 131,072], 50 steps
    python -m flowunsteady_gb300.runs large     # N = 1,048,576 helical wake (12 turns), 20 RK3 steps
    python -m flowunsteady_gb300.runs step      # k full steps of an N-particle wake (profiling)

They use the public API only (the C ABI through `_lib`, and `FieldBatch`).  Their
FP64 reference is the GPU FP64 direct sum, which the tests tie to the CPU oracle.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import sys
import time

import numpy as np

from . import _lib as L
from .batch import FieldBatch
from .workloads import batch_sizes, helical_wake, leapfrog_rings, uniform_box


class Field:
    """Minimal context wrapper over the C ABI."""

    def __init__(self, X, G, S, device=0, capacity=None):
        self.lib = L.lib()
        self.p = ctypes.c_void_p()
        n = X.shape[0]
        L.check(self.lib.vpm_ctx_create(device, capacity or n, ctypes.byref(self.p)))
        self.n = n
        self.set(X, G, S)

    def set(self, X, G, S):
        X, G, S = (np.ascontiguousarray(a, dtype=np.float64) for a in (X, G, S))
        L.check(self.lib.vpm_set_particles(self.p, X.shape[0], L.dptr(X), 3, L.dptr(G), 3,
                                           L.dptr(S), 1), self.p)

    def uj(self, kernel, prec, t0=0, t1=None):
        t1 = self.n if t1 is None else t1
        L.check(self.lib.vpm_eval_UJ_targets(self.p, kernel, prec, t0, t1), self.p)
        m = t1 - t0
        U, J = np.empty((m, 3)), np.empty((m, 3, 3))
        L.check(self.lib.vpm_get_UJ(self.p, t0, m, L.dptr(U), 3, L.dptr(J), 9), self.p)
        return U, J

    def step(self, scheme, dt, nsteps):
        L.check(self.lib.vpm_step(self.p, dt, ctypes.byref(scheme), nsteps, 1), self.p)

    def state(self):
        X, G, S = np.empty((self.n, 3)), np.empty((self.n, 3)), np.empty(self.n)
        L.check(self.lib.vpm_get_state(self.p, self.n, L.dptr(X), 3, L.dptr(G), 3, L.dptr(S), 1),
                self.p)
        return X, G, S

    def diag(self, kernel, prec):
        out = np.zeros(L.DIAG_COUNT)
        L.check(self.lib.vpm_diagnostics(self.p, kernel, prec, L.dptr(out)), self.p)
        return dict(zip(L.DIAG_NAMES, out.tolist()))

    def centroids(self, ranges):
        st = (ctypes.c_int64 * len(ranges))(*[r[0] for r in ranges])
        en = (ctypes.c_int64 * len(ranges))(*[r[1] for r in ranges])
        out = np.zeros((len(ranges), 3))
        L.check(self.lib.vpm_centroids(self.p, len(ranges), st, en, L.dptr(out)), self.p)
        return out

    def close(self):
        if self.p:
            self.lib.vpm_ctx_destroy(self.p)
            self.p = None


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def stretching(J, G):
    return np.einsum("iba,ib->ia", J, G)


def scheme_for(kernel, prec, sfs=L.SFS_DYNAMIC, nu=1e-4, rlxf=1.0, analytic=True):
    s = L.default_scheme()
    s.kernel, s.precision = kernel, prec
    s.sfs = sfs
    s.sfs_flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE
    if analytic:
        s.sfs_flags |= L.SFS_ANALYTIC_DSIGMA
    s.sfs_alpha, s.sfs_rlxf, s.sfs_minC, s.sfs_maxC = 0.999, rlxf, 0.0, 1.0
    s.nu = nu
    return s


def timed(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


# ------------------------------------------------------------- precision sweep --
def run_sweep(args):
    """U, J and stretching of FP32 and FP32C against FP64 (all GPU; the FP64
    kernel matches the CPU oracle to 1e-12), both kernels, N = 262,144."""
    n = args.n or 262144
    X, G, S = helical_wake(n)
    f = Field(X, G, S)
    res = {"workload": f"helical wake N={n}", "pairs": n * n, "kernels": {}}
    for kname, k in (("winckelmans", L.KERNEL_WINCKELMANS), ("gaussianerf", L.KERNEL_GAUSSIANERF)):
        (U64, J64), t64 = timed(lambda: f.uj(k, L.PREC_FP64))
        S64 = stretching(J64, G)
        row = {"fp64_s": t64, "fp64_pairs_per_s": n * n / t64}
        for pname, p in (("fp32", L.PREC_FP32), ("fp32c", L.PREC_FP32C)):
            f.uj(k, p)
            (U, J), t = timed(lambda: f.uj(k, p))
            row[pname] = {"seconds": t, "pairs_per_s": n * n / t, "rel_l2_U": rel_l2(U, U64),
                          "rel_l2_J": rel_l2(J, J64),
                          "rel_l2_stretching": rel_l2(stretching(J, G), S64)}
        res["kernels"][kname] = row
    f.close()
    return res


# ----------------------------------------------------------------------- rings --
def ring_observables(f, kernel, prec, nhalf):
    d = f.diag(kernel, prec)
    X, G, S = f.state()
    out = {"t_centroid_z": [], "radius": []}
    for lo, hi in ((0, nhalf), (nhalf, 2 * nhalf)):
        w = np.linalg.norm(G[lo:hi], axis=1)
        c = (w[:, None] * X[lo:hi]).sum(0) / w.sum()
        rad = (w * np.hypot(X[lo:hi, 0], X[lo:hi, 1])).sum() / w.sum()
        out["t_centroid_z"].append(float(c[2]))
        out["radius"].append(float(rad))
    out.update({"impulse_z": d["impulse_z"], "enstrophy": d["enstrophy"],
                "cd_mean": d["cd_mean"], "cd_zero_ratio": d["cd_zero_ratio"],
                "sigma_mean": d["sigma_mean"]})
    return out


def run_rings(args):
    """Two coaxial leapfrogging rings: Gaussian-erf, rVPM transposed, dynamic SFS
    with backscatter clipping, core spreading ν=1e-4, RK3 dt=0.005, 400 steps.
    FP64 and FP32C on the GPU from the same state."""
    X, G, S = leapfrog_rings()
    n = X.shape[0]
    nh = n // 2
    nsteps = args.steps or 400
    every = max(1, nsteps // 20)
    k = L.KERNEL_GAUSSIANERF
    res = {"workload": "leapfrogging rings, 2 x 200 x 19 = 7,600 particles", "n": n,
           "dt": 0.005, "steps": nsteps, "runs": {}}
    finals = {}
    for pname, p, an in (("fp64", L.PREC_FP64, False), ("fp32c", L.PREC_FP32C, False),
                         ("fp64_analytic", L.PREC_FP64, True),
                         ("fp32c_analytic", L.PREC_FP32C, True)):
        f = Field(X, G, S)
        sc = scheme_for(k, p, analytic=an)
        hist = [{"step": 0, **ring_observables(f, k, L.PREC_FP64, nh)}]
        t_run = 0.0
        for s0 in range(0, nsteps, every):
            m = min(every, nsteps - s0)
            _, t = timed(lambda: f.step(sc, 0.005, m))
            t_run += t
            hist.append({"step": s0 + m, **ring_observables(f, k, L.PREC_FP64, nh)})
        res["runs"][pname] = {"history": hist, "seconds_stepping": t_run,
                              "steps_per_s": nsteps / t_run}
        res["runs"][pname]["final_state"] = [a.tolist() for a in f.state()] if args.keep else None
        finals[pname] = f.state()
        f.close()

    def cmp(a, b):
        (Xa, Ga, Sa), (Xb, Gb, Sb) = finals[a], finals[b]
        return {"max_abs_dx": float(np.abs(Xa - Xb).max()), "rel_l2_gamma": rel_l2(Ga, Gb),
                "max_abs_dsigma": float(np.abs(Sa - Sb).max()), "rel_l2_sigma": rel_l2(Sa, Sb),
                "median_abs_dsigma": float(np.median(np.abs(Sa - Sb)))}

    res["fp32c_vs_fp64_final"] = cmp("fp32c", "fp64")
    res["fp32c_analytic_vs_fp64_analytic_final"] = cmp("fp32c_analytic", "fp64_analytic")
    res["fp64_analytic_vs_fp64_final"] = cmp("fp64_analytic", "fp64")
    return res


# ----------------------------------------------------------------------- batch --
def run_batch(args):
    """48 independent fields (uniform-box distribution, N_i log-uniform in
    [2,048, 131,072]), FP32C, Gaussian-erf with dynamic SFS: every pair pass of
    a stage is one persistent launch over all fields and every step is one
    graph replay; 50 steps are timed.  Checks: one batched U/J evaluation
    against 48 separate FP64 evaluations, and the 50-step trajectories of the
    six smallest fields against separate FP64 contexts."""
    sizes = [int(v) for v in batch_sizes(args.fields or 48)]
    nsteps = args.steps or 50
    fields = []
    for f, n in enumerate(sizes):
        X, G, S = uniform_box(n, seed_index=1000 + f)
        fields.append((X, G * 10.0, S))
    k = L.KERNEL_GAUSSIANERF
    sc = scheme_for(k, L.PREC_FP32C)
    b = FieldBatch(sizes)

    def load():
        for f, (X, G, S) in enumerate(fields):
            b.set_field(f, X, G, S)

    load()
    tuned_ms = b.autotune(k, L.PREC_FP32C) if args.autotune else None
    b.eval_UJ(k, L.PREC_FP32C)
    shapes = sorted({f"{bl}x{tp}" for bl, tp in b.shapes()})
    (_, t_uj) = timed(lambda: b.eval_UJ(k, L.PREC_FP32C))
    uj = [b.get_UJ(f) for f in range(len(sizes))]
    b.step(0.005, sc, 1)                       # capture + warm-up
    load()                                     # restart from the initial state
    _, t_batch = timed(lambda: b.step(0.005, sc, nsteps))
    got = [b.get_field(f) for f in range(len(sizes))]
    b.close()
    pairs_step = sum(n * n for n in sizes)
    res = {"workload": f"{len(sizes)} fields, N in [{min(sizes)}, {max(sizes)}]",
           "sizes": sizes, "sum_n": sum(sizes), "sum_n2": pairs_step, "steps": nsteps,
           "tile_shapes": shapes, "autotuned": bool(args.autotune), "autotune_uj_ms": tuned_ms,
           "batch_uj_seconds": t_uj, "batch_uj_pairs_per_s": pairs_step / t_uj,
           "batch_seconds": t_batch, "batch_steps_per_s": nsteps / t_batch,
           # dynamic SFS: stage 1 runs U/J and ζ at σ and ασ, stages 2-3 once: 4 U/J passes
           "uj_pairs_per_s_in_steps": 4 * pairs_step * nsteps / t_batch}
    if not args.no_reference:
        eu, ej, t64 = [], [], 0.0
        for f, (X, G, S) in enumerate(fields):
            fl = Field(X, G, S)
            (U0, J0), t = timed(lambda: fl.uj(k, L.PREC_FP64))
            t64 += t
            fl.close()
            if X.shape[0] > 1:
                eu.append(rel_l2(uj[f][0], U0))
                ej.append(rel_l2(uj[f][1], J0))
        res["uj_fp32c_batch_vs_separate_fp64"] = {"max_rel_l2_U": max(eu), "max_rel_l2_J": max(ej),
                                                  "fp64_seconds": t64}
        sc64 = scheme_for(k, L.PREC_FP64)
        small = sorted(range(len(sizes)), key=lambda f: sizes[f])[:6]
        dx, dg, ds = [], [], []
        for f in small:
            X, G, S = fields[f]
            fl = Field(X, G, S)
            fl.step(sc64, 0.005, nsteps)
            Xr, Gr, Sr = fl.state()
            fl.close()
            Xb, Gb, Sb = got[f]
            dx.append(float(np.abs(Xb - Xr).max()))
            dg.append(rel_l2(Gb, Gr))
            ds.append(float(np.abs(Sb - Sr).max()))
        res["steps_fp32c_batch_vs_separate_fp64_smallest6"] = {
            "fields": small, "max_abs_dx": max(dx), "max_rel_l2_gamma": max(dg),
            "max_abs_dsigma": max(ds)}
    return res


# ----------------------------------------------------------------------- large --
def run_large(args):
    """N = 1,048,576 helical wake with 12 turns: 20 RK3 steps of full rVPM
    (Gaussian-erf, dynamic SFS, core spreading ν=1e-4, dt=0.002) with FP32C pair
    passes; after every step U/J at 4,096 seeded sampled targets are checked
    against the FP64 direct sum of the same state."""
    n = args.n or 1048576
    nsteps = args.steps or 20
    dt = args.dt or 0.002
    X, G, S = helical_wake(n, turns=12)
    f = Field(X, G, S)
    k = L.KERNEL_GAUSSIANERF
    sc = scheme_for(k, L.PREC_FP32C)
    rng = np.random.default_rng(20261207)
    checks = []
    t_steps = 0.0
    import torch
    dev = torch.device("cuda:0")
    for s in range(nsteps):
        _, t = timed(lambda: f.step(sc, dt, 1))
        t_steps += t
        Xs, Gs, Ss = f.state()
        idx = np.sort(rng.choice(n, 4096, replace=False))
        Xd = torch.tensor(Xs.T.copy(), device=dev)
        Gd = torch.tensor(Gs.T.copy(), device=dev)
        Sd = torch.tensor(Ss, device=dev)
        Td = torch.tensor(Xs[idx].T.copy(), device=dev)
        outs = {}
        for p in (L.PREC_FP64, L.PREC_FP32C):
            U = torch.empty((3, 4096), dtype=torch.float64, device=dev)
            J = torch.empty((9, 4096), dtype=torch.float64, device=dev)
            L.check(L.lib().vpm_uj_device_async(k, p, n, Xd.data_ptr(), Gd.data_ptr(), Sd.data_ptr(),
                                                n, 4096, Td.data_ptr(), 4096, U.data_ptr(),
                                                J.data_ptr(), 4096, None))
            torch.cuda.synchronize()
            outs[p] = (U.cpu().numpy().T, J.cpu().numpy().T.reshape(4096, 3, 3))
        U64, J64 = outs[L.PREC_FP64]
        U32, J32 = outs[L.PREC_FP32C]
        checks.append({"step": s + 1, "step_seconds": t, "rel_l2_U": rel_l2(U32, U64),
                       "rel_l2_J": rel_l2(J32, J64),
                       "rel_l2_stretching": rel_l2(stretching(J32, Gs[idx]), stretching(J64, Gs[idx]))})
    d = f.diag(k, L.PREC_FP32C)
    f.close()
    return {"workload": f"helical wake N={n}, 12 turns", "steps": nsteps, "dt": dt,
            "seconds_stepping": t_steps, "seconds_per_step": t_steps / nsteps,
            "uj_pairs_per_step": 4 * n * n, "checks": checks,
            "max_rel_l2_U": max(c["rel_l2_U"] for c in checks),
            "max_rel_l2_J": max(c["rel_l2_J"] for c in checks), "final_diagnostics": d}


# ------------------------------------------------------------------------- fmm --
def run_fmm(args):
    """Treecode (vpm_eval_UJ_fmm, FLOWUnsteady's default settings p=4,
    ncrit=50, θ=0.4) against the direct FP32C sum on a helical wake: time per
    evaluation of both, and the FP32C/FP64 accuracy of both on 4,096 sampled
    targets against the GPU FP64 direct sum."""
    import torch
    n = args.n or 1048576
    X, G, S = helical_wake(n, turns=12 if n > 500000 else 4)
    f = Field(X, G, S)
    k = L.KERNEL_GAUSSIANERF
    fm = L.default_fmm()
    if args.local_order is not None:
        fm.local_order = args.local_order
    if args.fmm_p is not None:
        fm.p = args.fmm_p
    if args.theta is not None:
        fm.theta = args.theta
    L.check(f.lib.vpm_eval_UJ_fmm(f.p, k, L.PREC_FP32C, ctypes.byref(fm)), f.p)   # warm-up
    ts = []
    for _ in range(3):
        _, t = timed(lambda: L.check(f.lib.vpm_eval_UJ_fmm(f.p, k, L.PREC_FP32C, ctypes.byref(fm)), f.p))
        ts.append(t)
    st = (ctypes.c_int64 * len(L.FMM_STATS))()
    L.check(f.lib.vpm_fmm_stats(f.p, st), f.p)
    stats = dict(zip(L.FMM_STATS, st))
    Uf, Jf = np.empty((n, 3)), np.empty((n, 3, 3))
    L.check(f.lib.vpm_get_UJ(f.p, 0, n, L.dptr(Uf), 3, L.dptr(Jf), 9), f.p)
    _, t_direct = timed(lambda: L.check(f.lib.vpm_eval_UJ(f.p, k, L.PREC_FP32C), f.p))
    Ud, Jd = np.empty((n, 3)), np.empty((n, 3, 3))
    L.check(f.lib.vpm_get_UJ(f.p, 0, n, L.dptr(Ud), 3, L.dptr(Jd), 9), f.p)
    f.close()
    rng = np.random.default_rng(20261207)
    idx = np.sort(rng.choice(n, 4096, replace=False))
    dev = torch.device("cuda:0")
    Xd = torch.tensor(X.T.copy(), device=dev)
    Gd = torch.tensor(G.T.copy(), device=dev)
    Sd = torch.tensor(S, device=dev)
    Td = torch.tensor(X[idx].T.copy(), device=dev)
    U = torch.empty((3, 4096), dtype=torch.float64, device=dev)
    J = torch.empty((9, 4096), dtype=torch.float64, device=dev)
    L.check(L.lib().vpm_uj_device_async(k, L.PREC_FP64, n, Xd.data_ptr(), Gd.data_ptr(),
                                        Sd.data_ptr(), n, 4096, Td.data_ptr(), 4096, U.data_ptr(),
                                        J.data_ptr(), 4096, None))
    torch.cuda.synchronize()
    U64, J64 = U.cpu().numpy().T, J.cpu().numpy().T.reshape(4096, 3, 3)
    return {"workload": f"helical wake N={n}", "kernel": "gaussianerf", "precision": "fp32c",
            "fmm": {"p": fm.p, "ncrit": fm.ncrit, "theta": fm.theta,
                    "sigma_factor": fm.sigma_factor, "local_order": fm.local_order},
            "seconds_fmm": min(ts), "seconds_direct": t_direct,
            "speedup": t_direct / min(ts),
            **stats,
            "near_sources_per_target": stats["near_pairs"] / n,
            "far_cells_per_target": stats["far_evaluations"] / n,
            "local_cells_per_group": stats["local_terms"] / max(stats["groups"], 1),
            "fmm_rel_l2_U": rel_l2(Uf[idx], U64), "fmm_rel_l2_J": rel_l2(Jf[idx], J64),
            "direct_rel_l2_U": rel_l2(Ud[idx], U64), "direct_rel_l2_J": rel_l2(Jd[idx], J64)}


# -------------------------------------------------------------------- treestep --
def run_treestep(args):
    """The same helical wake stepped twice from one state: U/J and analytic
    dynamic-SFS passes by the treecode (vpm_scheme.uj_method = VPM_UJ_TREE,
    p=4, ncrit=50, θ=0.4) and by the direct FP32C sum; time per step of both and
    the distance of the two trajectories after every step."""
    n = args.n or 1048576
    nsteps = args.steps or 10
    dt = args.dt or 1e-4
    X, G, S = helical_wake(n, turns=12 if n > 500000 else 4)
    sd = scheme_for(L.KERNEL_GAUSSIANERF, L.PREC_FP32C)
    st = scheme_for(L.KERNEL_GAUSSIANERF, L.PREC_FP32C)
    st.uj_method = L.UJ_TREE
    st.fmm = L.default_fmm()
    fd, ft = Field(X, G, S), Field(X, G, S)
    hist, td, tt = [], 0.0, 0.0
    for k in range(nsteps):
        _, a = timed(lambda: fd.step(sd, dt, 1))
        _, b = timed(lambda: ft.step(st, dt, 1))
        td += a
        tt += b
        Xd, Gd, Sd = fd.state()
        Xt, Gt, St = ft.state()
        hist.append({"step": k + 1, "max_abs_dx": float(np.abs(Xt - Xd).max()),
                     "rel_l2_gamma": rel_l2(Gt, Gd), "rel_max_sigma": float(np.abs(St - Sd).max() / np.abs(Sd).max())})
    dg = ft.diag(L.KERNEL_GAUSSIANERF, L.PREC_FP32C)
    fd.close()
    ft.close()
    return {"workload": f"helical wake N={n}, dynamic SFS (analytic), nu=1e-4", "dt": dt,
            "steps": nsteps, "seconds_per_step_direct": td / nsteps,
            "seconds_per_step_tree": tt / nsteps, "speedup": td / tt, "history": hist,
            "final_sigma_mean": dg["sigma_mean"], "final_nonfinite": dg["nonfinite"]}


# ------------------------------------------------------------------------ step --
def run_step(args):
    """k full RK3 steps (Gaussian-erf, dynamic SFS with analytic ∂/∂σ, ν = 1e-4,
    FP32C pair passes) of an N-particle helical wake; a plain driver for
    profiling the O(N) kernels at sizes above L2."""
    n = args.n or 1048576
    nsteps = args.steps or 1
    X, G, S = helical_wake(n, turns=12 if n > 500000 else 4)
    f = Field(X, G, S)
    sc = scheme_for(L.KERNEL_GAUSSIANERF, L.PREC_FP32C)
    if args.tree:
        sc.uj_method = L.UJ_TREE
        sc.fmm = L.default_fmm()
    tuned = None
    if args.autotune:
        tile, ms = L.Tile(), ctypes.c_double()
        L.check(f.lib.vpm_autotune(f.p, L.KERNEL_GAUSSIANERF, L.PREC_FP32C, ctypes.byref(tile),
                                   ctypes.byref(ms)), f.p)
        tuned = {"uj": f"{tile.block}x{tile.tpt}", "zeta": "{}x{}".format(*divmod(tile.reserved, 16))}
    _, t = timed(lambda: f.step(sc, args.dt or 1e-4, nsteps))
    d = f.diag(L.KERNEL_GAUSSIANERF, L.PREC_FP32C)
    f.close()
    return {"workload": f"helical wake N={n}", "steps": nsteps, "seconds": t,
            "seconds_per_step": t / nsteps, "tile": tuned,
            "uj": "treecode p4 ncrit50 theta0.4" if args.tree else "direct",
            "sigma_mean": d["sigma_mean"], "nonfinite": d["nonfinite"]}


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("run", choices=["sweep", "rings", "batch", "large", "step", "fmm", "treestep"])
    p.add_argument("--n", type=int, default=None)
    p.add_argument("--steps", type=int, default=None)
    p.add_argument("--fields", type=int, default=None)
    p.add_argument("--dt", type=float, default=None)
    p.add_argument("--keep", action="store_true", help="include the final state (rings)")
    p.add_argument("--no-reference", action="store_true", help="batch: skip the FP64 fields")
    p.add_argument("--autotune", action="store_true",
                   help="step, batch: tune the tile shapes first (per size bucket for a batch)")
    p.add_argument("--tree", action="store_true", help="step: U/J passes by the treecode")
    p.add_argument("--local-order", type=int, default=None,
                   help="fmm: treecode local expansion order (0: M2P only)")
    p.add_argument("--fmm-p", type=int, default=None, help="fmm: expansion order of the moments")
    p.add_argument("--theta", type=float, default=None, help="fmm: acceptance parameter")
    p.add_argument("--out", default=None)
    args = p.parse_args(argv)
    fn = {"sweep": run_sweep, "rings": run_rings, "batch": run_batch, "large": run_large,
          "step": run_step, "fmm": run_fmm, "treestep": run_treestep}[args.run]
    res = fn(args)
    txt = json.dumps(res)
    if args.out:
        with open(args.out, "w") as fh:
            fh.write(txt + "\n")
    print(txt if len(txt) < 4000 else txt[:4000] + " ...")


if __name__ == "__main__":
    main()
