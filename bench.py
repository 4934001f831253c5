#!/usr/bin/env python
"""Benchmark of the rVPM U+∇U pair pass on GB300.

Workload: the helical-wake precision-sweep field, N = 262,144 particles (90 %
on three helices of radius 1, pitch 0.2, 4 turns with N(0, 0.01) jitter, Γ
tangent with |Γ| = 1/√N_helix; 10 % uniform in [-1.5,1.5]³ with Γ ~ N(0,1e-4);
σ = 0.03), seeded synthetic data.  One step = one FP32-compensated U and ∇U
evaluation at every particle from every particle (N² pair interactions) with
the Gaussian-erf kernel, FLOWUnsteady's default.

Metric: pair interactions per second.  `value` is device time of the
evaluation with the particle field resident in HBM; `e2e` is the same metric
through the C ABI with host arrays (upload of X, Γ, σ and download of U, J
inside the timed region, every step).  The accuracy of the timed run (relative
L2 of U, J and the stretching term against the CPU FP64 oracle on the targets
the CPU baseline sampled) and the GPU FP64 throughput on the same targets are
reported beside it.

`--impl reference` times the CPU FP64 restatement of the pair sum (the
checker in oracle/, OpenMP over all host cores) on a bounded target sample of
the same workload: FLOWVPM's own UJ_direct (Julia) cannot run on this machine.

Multi-GPU: the pair pass does not shard here (one GPU per box); `--gpus N`
under torchrun runs N independent replicas (weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PAIR_FLOP = 60          # algorithmic flop per U+∇U pair (FMA = 2)
BYTES_H2D = 56          # X, Γ, σ per particle (FP64)
BYTES_D2H = 96          # U (3) and J (9) per particle (FP64)
L2_FLUSH_BYTES = 256 << 20
# DRAM bytes (read + write) of one Gaussian-erf FP32C U/J launch of the
# benchmark workload per (N, tile shape), from an ncu capture.  The plain U/J
# pass is split into about 64 waves of short work items (57 source chunks per
# target tile with 128x4), which measured 5 % faster than whole tiles.  The
# last CTA of each tile sums the chunks' partial sums from L2 and drops
# them there; what still reaches DRAM is partial sums evicted before their tile
# was complete.  (With a separate reduction launch the partial sums took 1.8 GB.)
PAIR_KERNEL_TRAFFIC = {(262144, "128x4"): 64656640 + 138696448}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--kernel", default="gaussianerf", choices=["gaussianerf", "winckelmans"])
    p.add_argument("--n", type=int, default=262144)
    p.add_argument("--sample-targets", type=int, default=8192)
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--precision", default="fp32c", choices=["fp32c", "fp32", "fp64"])
    p.add_argument("--tile", default=None,
                   help="pin the pair-kernel tile shape, e.g. 128x4 (default: autotuner/default)")
    p.add_argument("--timed-only", action="store_true",
                   help="run only the warm-up and timed evaluations (for profiler captures)")
    return p.parse_args()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def workload_config(args):
    """The workload description shared by both arms (precision is per arm)."""
    return {"workload": f"helical wake N={args.n}, one U+∇U evaluation at every particle, "
                        f"{args.kernel} kernel",
            "n_particles": args.n, "pairs_per_step": args.n * args.n}


def aggregate(total_s, steps, pairs_per_step, world, dist, device=None):
    """Whole-job pairs/s: every rank runs its own replica; the job takes the
    slowest rank's time (max over ranks)."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([float(total_s)], dtype=torch.float64,
                         device=device if device is not None else "cpu")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())
    return world * steps * pairs_per_step / total_s, total_s


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local, dist


def cpu_pair_rate(X, G, S, kernel, seconds, seed=7, keep=None):
    """Pairs/s of the CPU FP64 direct sum (oracle, all host threads) on a
    target sample sized to about `seconds` of work.  When `keep` is a dict it
    receives the sample's indices and the oracle's U and J there."""
    from oracle import oracle as O
    O.build()
    rng = np.random.default_rng(seed)
    n = X.shape[0]
    m = 64
    t = 0.0
    while True:
        idx = rng.choice(n, m, replace=False)
        t0 = time.perf_counter()
        O.uj_direct(kernel, X, G, S, Xt=X[idx])
        t = time.perf_counter() - t0
        if t >= 0.5 or m >= n:
            break
        m = min(n, m * 4)
    rate = m * n / t
    m_final = int(min(n, max(m, rate * seconds / n)))
    idx = np.sort(rng.choice(n, m_final, replace=False))
    t0 = time.perf_counter()
    U, J = O.uj_direct(kernel, X, G, S, Xt=X[idx])
    t = time.perf_counter() - t0
    if keep is not None:
        keep.update(idx=idx, U=U, J=J)
    return m_final * n / t, m_final, t, O.max_threads()


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def run_reference(args, world, rank):
    from flowunsteady_gb300.workloads import helical_wake
    if rank != 0:
        return
    kernel = 1 if args.kernel == "gaussianerf" else 0
    X, G, S = helical_wake(args.n)
    # Each step: a bounded target sample against all N sources.
    rate0, m, _, cores = cpu_pair_rate(X, G, S, kernel, min(args.cpu_seconds, 5.0))
    from oracle import oracle as O
    rng = np.random.default_rng(11)
    m_step = int(max(64, min(args.n, rate0 * 2.0 / args.n)))  # ~2 s per step
    for _ in range(args.warmup):
        O.uj_direct(kernel, X, G, S, Xt=X[rng.choice(args.n, 64, replace=False)])
    times = []
    for _ in range(args.steps):
        idx = rng.choice(args.n, m_step, replace=False)
        t0 = time.perf_counter()
        O.uj_direct(kernel, X, G, S, Xt=X[idx])
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = args.steps * m_step * args.n / total
    sample = (f"{m_step} random targets x {args.n} sources per step, helical wake, "
              f"{args.kernel}, FP64, OpenMP {cores} threads on {cpu_model()}")
    line = {
        "impl": "reference",
        "metric": "U+∇U pair-interactions/s",
        "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic (seeded helical wake, {args.n} particles)",
        "config": {**workload_config(args), "precision": "fp64 (CPU)"},
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "FLOWVPM UJ_direct (Julia) is not runnable here (Julia absent, FLOWVPM not "
                "vendored); the arm times the CPU FP64 restatement of the same pair sum.",
    }
    print(json.dumps(line))


def run_ours(args, world, rank, local, dist):
    import torch
    from flowunsteady_gb300 import _lib as L
    from flowunsteady_gb300.workloads import helical_wake

    lib = L.lib()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    kernel = L.KERNEL_GAUSSIANERF if args.kernel == "gaussianerf" else L.KERNEL_WINCKELMANS
    n = args.n
    X, G, S = helical_wake(n)
    X, G, S = (np.ascontiguousarray(a) for a in (X, G, S))

    f32 = ctypes.c_double()
    f64 = ctypes.c_double()
    mhz = ctypes.c_double()
    if not args.timed_only:
        L.check(lib.vpm_measure_fma_peaks(local, ctypes.byref(f32), ctypes.byref(f64),
                                          ctypes.byref(mhz)))

    ctx = ctypes.c_void_p()
    L.check(lib.vpm_ctx_create(local, n, ctypes.byref(ctx)))
    stream = torch.cuda.current_stream(dev)
    L.check(lib.vpm_ctx_set_stream(ctx, ctypes.c_void_p(stream.cuda_stream)), ctx)
    L.check(lib.vpm_set_particles(ctx, n, L.dptr(X), 3, L.dptr(G), 3, L.dptr(S), 1), ctx)
    if args.tile:
        b_, t_ = (int(v) for v in args.tile.lower().split("x"))
        tile = L.Tile(b_, t_, 0, 0)
        L.check(lib.vpm_set_tile(ctx, kernel, {"fp32c": L.PREC_FP32C, "fp32": L.PREC_FP32,
                                               "fp64": L.PREC_FP64}[args.precision],
                                 ctypes.byref(tile)), ctx)
    prec = {"fp32c": L.PREC_FP32C, "fp32": L.PREC_FP32, "fp64": L.PREC_FP64}[args.precision]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    tuned = None
    if not args.tile and not args.timed_only:
        # Tile shape for this size bucket from the autotuner (one timed
        # evaluation per compiled shape); later evaluations use it.
        tile, tms = L.Tile(), ctypes.c_double()
        L.check(lib.vpm_autotune(ctx, kernel, prec, ctypes.byref(tile), ctypes.byref(tms)), ctx)
        tuned = f"{tile.block}x{tile.tpt}"
    for _ in range(args.warmup):
        L.check(lib.vpm_eval_UJ(ctx, kernel, prec), ctx)
    torch.cuda.synchronize(dev)

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    l0 = ctypes.c_int64()
    l1 = ctypes.c_int64()
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    lib.vpm_get_launch_count(ctx, ctypes.byref(l0))
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.fill_(float(k))            # evict L2 between timed steps
            starts[k].record(stream)
            L.check(lib.vpm_eval_UJ(ctx, kernel, prec), ctx)
            ends[k].record(stream)
        torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    lib.vpm_get_launch_count(ctx, ctypes.byref(l1))
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    pairs = float(n) * float(n)
    value, total_s = aggregate(sum(step_ms) / 1e3, args.steps, pairs, world, dist, dev)
    ms_per_step = 1e3 * total_s / args.steps
    launches = int(l1.value - l0.value)
    # The other kernel, timed the same way (reported beside the headline).
    other = None
    if not args.timed_only:
        k2 = L.KERNEL_WINCKELMANS if kernel == L.KERNEL_GAUSSIANERF else L.KERNEL_GAUSSIANERF
        tile2, tms2 = L.Tile(), ctypes.c_double()
        L.check(lib.vpm_autotune(ctx, k2, prec, ctypes.byref(tile2), ctypes.byref(tms2)), ctx)
        for _ in range(2):
            L.check(lib.vpm_eval_UJ(ctx, k2, prec), ctx)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        for k in range(args.steps):
            flush.fill_(float(k))
            ev[k][0].record(stream)
            L.check(lib.vpm_eval_UJ(ctx, k2, prec), ctx)
            ev[k][1].record(stream)
        torch.cuda.synchronize(dev)
        ms2 = sum(a.elapsed_time(b) for a, b in ev) / args.steps
        other = {"kernel": "winckelmans" if k2 == L.KERNEL_WINCKELMANS else "gaussianerf",
                 "ms_per_step": ms2, "pairs_per_s": float(n) * n / (ms2 / 1e3),
                 "tile": f"{tile2.block}x{tile2.tpt}",
                 "frac_of_fp32_fma_peak": (PAIR_FLOP * float(n) * n / (ms2 / 1e3) / 1e12 / f32.value
                                           if f32.value > 0 else None)}
    if args.timed_only:
        if rank == 0:
            print(json.dumps({"timed_only": True, "ms_per_step": ms_per_step,
                              "pairs_per_s": value, "gpu_launches": launches, "tile": args.tile,
                              "kernel": args.kernel, "precision": args.precision, "n": n}))
        lib.vpm_ctx_destroy(ctx)
        return None

    # ---- end to end through the C ABI with host buffers ------------------------
    # As many steps as the device-timed region; each uploads X, Γ, σ from host
    # arrays, evaluates and downloads U, J (host clock around the whole step).
    U = np.empty((n, 3))
    J = np.empty((n, 9))
    e2e_t = []
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        L.check(lib.vpm_set_particles(ctx, n, L.dptr(X), 3, L.dptr(G), 3, L.dptr(S), 1), ctx)
        L.check(lib.vpm_eval_UJ(ctx, kernel, prec), ctx)
        L.check(lib.vpm_get_UJ(ctx, 0, n, L.dptr(U), 3, L.dptr(J), 9), ctx)
        e2e_t.append(time.perf_counter() - t0)
    e2e_value, _ = aggregate(sum(e2e_t), args.steps, pairs, world, dist, dev)

    # ---- CPU baseline; its target sample doubles as the accuracy reference -----
    cpu = None
    ref = {}
    if rank == 0 and world == 1:
        rate, mt, tt, cores = cpu_pair_rate(X, G, S, kernel, args.cpu_seconds, keep=ref)
        cpu = {"value": rate, "unit": "pairs/s", "cores": cores, "kind": "port",
               "sample": f"{mt} random targets x {n} sources ({tt:.1f} s), FP64 oracle, "
                         f"OpenMP on {cpu_model()}"}

    # ---- accuracy of the timed result and FP64 throughput on sampled targets ---
    if ref:
        idx = ref["idx"]
    else:
        rng = np.random.default_rng(2026)
        idx = np.sort(rng.choice(n, min(args.sample_targets, n), replace=False))
    m = idx.size
    Xs_d = torch.tensor(X.T.copy(), device=dev)
    Gs_d = torch.tensor(G.T.copy(), device=dev)
    Ss_d = torch.tensor(S, device=dev)
    Xt_d = torch.tensor(X[idx].T.copy(), device=dev)
    out = {}
    for p in (L.PREC_FP64, L.PREC_FP32C):
        Ud = torch.empty((3, m), dtype=torch.float64, device=dev)
        Jd = torch.empty((9, m), dtype=torch.float64, device=dev)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        for rep in range(2):
            ev0.record(stream)
            rc = lib.vpm_uj_device_async(kernel, p, n, Xs_d.data_ptr(), Gs_d.data_ptr(),
                                         Ss_d.data_ptr(), n, m, Xt_d.data_ptr(), m,
                                         Ud.data_ptr(), Jd.data_ptr(), m,
                                         ctypes.c_void_p(stream.cuda_stream))
            ev1.record(stream)
            L.check(rc)
        torch.cuda.synchronize(dev)
        out[p] = (Ud.cpu().numpy().T, Jd.cpu().numpy().T.reshape(m, 3, 3),
                  ev0.elapsed_time(ev1) / 1e3)
    U64, J64, t64 = out[L.PREC_FP64]
    fp64_rate = m * float(n) / t64
    Uf = U[idx]
    Jf = J[idx].reshape(m, 3, 3)
    S64 = np.einsum("iba,ib->ia", J64, G[idx])
    Sf = np.einsum("iba,ib->ia", Jf, G[idx])

    def rl2(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    if ref:
        # Against the CPU FP64 oracle; the GPU FP64 sum at the same targets too.
        Uo, Jo = ref["U"], ref["J"]
        So = np.einsum("iba,ib->ia", Jo, G[idx])
        acc = {"U": rl2(Uf, Uo), "J": rl2(Jf, Jo), "stretching": rl2(Sf, So),
               "fp64_U": rl2(U64, Uo), "fp64_J": rl2(J64, Jo),
               "reference": f"CPU FP64 oracle (oracle/) on {m} sampled targets"}
    else:
        acc = {"U": rl2(Uf, U64), "J": rl2(Jf, J64), "stretching": rl2(Sf, S64),
               "reference": f"GPU FP64 direct sum on {m} sampled targets"}

    # ---- roofline of the dominant kernel (the pair kernel) ------------------------
    achieved = PAIR_FLOP * pairs / (ms_per_step / 1e3) / 1e12
    roof = {"bound": "fp32_fma", "achieved": achieved, "peak": f32.value, "unit": "TFLOP/s",
            "frac": achieved / f32.value if f32.value > 0 else None,
            "traffic": PAIR_KERNEL_TRAFFIC.get((n, args.tile or tuned)),
            "traffic_unit": "bytes per launch (ncu dram__bytes_read + dram__bytes_write)",
            "peak_source": "in-repo FFMA microbenchmark (vpm_measure_fma_peaks) in this run",
            "fp64_peak_tflops": f64.value, "microbench_sm_mhz": mhz.value,
            "flop_per_pair": PAIR_FLOP}

    line = None
    if rank == 0:
        line = {
            "metric": "U+∇U pair-interactions/s",
            "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (compensated; FP64 state)",
            "data": "synthetic (seeded helical wake)",
            "config": {**workload_config(args), "precision": args.precision,
                       "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": BYTES_H2D * n,
                    "d2h_bytes_per_step": BYTES_D2H * n},
            "gpu_launches": launches,
            "roofline": roof,
            "cpu_baseline": cpu,
            "accuracy_rel_l2": acc,
            "fp64_pairs_per_s": fp64_rate,
            "fp32c_over_fp64": value / world / fp64_rate,
            "clocks": clk.summary(),
            "step_ms": step_ms,
            "tile": args.tile or tuned,
            "other_kernel": other,
        }
        print(json.dumps(line))
    lib.vpm_ctx_destroy(ctx)
    return line


def main():
    args = parse()
    world, rank, local, dist = dist_setup(args)
    try:
        if args.impl == "reference":
            run_reference(args, world, rank)
        else:
            run_ours(args, world, rank, local, dist)
    finally:
        if dist:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
