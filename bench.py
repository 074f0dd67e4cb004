"""Benchmark of the real-time lattice Yang-Mills hot path on GB300.

Workload (the configuration the headline metric is quoted on): SU(3)
Hamiltonian leapfrog on a 128^3 periodic lattice, dt = 0.05, FP32 storage
(two-row SU(3) links) with FP64 reunitarisation every 100 steps.  Synthetic
initial state: links exp(i theta^a t^a), theta ~ N(0, 0.3^2) (seed 2), E ~
N(0, 1/2) per component (seed 1), Gauss-restored in FP64.  One bench step is
one full leapfrog step = 3 * 128^3 link-updates.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm prints one JSON line with the device-resident throughput (`value`),
the end-to-end throughput through the C ABI with host buffers (`e2e`), the
roofline of the step kernel, the CPU baseline (the oracle on this host's
cores), clocks and the launch count.  The reference arm (--impl reference)
times the reference's CPU implementation of the same step on all host cores.
Under torchrun (N > 1) every rank runs an independent replica (no collective
on the data path): value = all ranks' link-updates / max-over-ranks time.
"""
from __future__ import annotations

import argparse
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

METRIC = "SU(3) link-updates/s @128^3"
UNIT = "link-updates/s"
# algorithmic bytes per link-update of the fused step, SU(3) FP32 two-row:
# links read once + written once (2 x 48 B), fields read once + written once (2 x 32 B)
BYTES_PER_LINK = 160
FALLBACK_HBM_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--size", type=int, default=128)
    p.add_argument("--dt", type=float, default=0.05)
    p.add_argument("--e2e-steps", type=int, default=10)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 path's sub-record")
    # other configurations of the reference's workload, each with its own JSON line:
    # ensemble = 256 mixed trajectories in batched launches; serve = Poisson request stream
    p.add_argument("--workload", default="leapfrog", choices=["leapfrog", "ensemble", "serve"])
    p.add_argument("--requests", type=int, default=100)
    p.add_argument("--serve-window", type=float, default=30.0,
                   help="seconds over which the sustainable serving rate is measured")
    p.add_argument("--trajectories", type=int, default=256)
    return p.parse_args()


def config(L, dt):
    """The workload, identical in both arms (what is computed, not how it is stored)."""
    return {
        "workload": f"SU(3) Hamiltonian leapfrog {L}^3, dt={dt}",
        "group": "SU(3)", "L": L, "dt": dt,
        "l2": "inputs larger than L2 (the 128^3 state is 805 MB in FP32 storage, 1.31 GB in the FP64 AoS layout)",
        "parallelism": "replicas (independent lattices per GPU)",
        "ic": "links exp(i theta t), theta~N(0,0.09) seed 2; E~N(0,0.5) seed 1; FP64 Gauss restore",
    }


def impl_config(L, tile):
    """How our arm stores and steps the workload."""
    return {"storage": "FP32 two-row SU(3) links (48 B) + FP32 fields (32 B) per link, site pairs packed",
            "reductions": "fp64", "reunitarisation": "FP64, every 100 steps", "tile": tile,
            "device": "one GPU"}


def reference_impl_config(cores):
    return {"storage": "FP64 AoS (the reference's GaugeLinks/ElectricFields layout)", "reductions": "fp64",
            "reunitarisation": "none (the reference never reunitarises)", "tile": "n/a (CPU, OpenMP over z)",
            "device": f"CPU, {cores} host threads"}


# ------------------------------------------------------------------ helpers
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, device):
    """x's maximum over the ranks of the default process group (x alone without one):
    each rank times its own replica, and the job takes as long as the slowest."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic():
    """DRAM bytes per launch of the step kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "step_su3_fp32_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get("dram_bytes_per_launch_scaled_128")
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks, load and throttle reasons, sampled every 200 ms by a
    read-only query from before the initial-state preparation to the end of the
    GPU work around the timed region (the timed region alone is a few ms)."""

    Q = ("clocks.sm,clocks.max.sm,utilization.gpu,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.marks = {}

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))

    def mark(self, name):
        self.marks[name] = time.monotonic()

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)  # one more sample after the last kernel
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.proc = None

    def summary(self):
        rows, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm, mx, util = float(parts[0]), float(parts[1]), float(parts[2])
            except ValueError:
                continue
            act = {n for n, v in zip(names, parts[4:8]) if v.lower().startswith("active")}
            rows.append((t, sm, util, act))
        loaded = [r for r in rows if r[2] >= 50.0]
        for r in loaded:
            reasons |= r[3]
        t0, t1 = self.marks.get("timed_start"), self.marks.get("timed_end")
        in_timed = [r for r in rows if t0 is not None and t0 - 0.2 <= r[0] <= t1 + 0.2]
        return {"sm_mhz": statistics.median([r[1] for r in loaded]) if loaded else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(rows), "samples_under_load": len(loaded),
                "samples_at_timed_region": len(in_timed),
                "window": "every 200 ms from the initial-state preparation (FP64 restore) through the timed region "
                          "and the FP64 comparison; under load = utilization.gpu >= 50%"}


# --------------------------------------------------------------- CPU timing
def cpu_leapfrog_rate(L, dt, min_seconds=10.0, max_steps=10, prefer_reference=True):
    """Reference CPU implementation (oracle/_ref where it was compiled on this
    host, else the oracle's restatement) on all host cores: link-updates/s."""
    import oracle
    cores = os.cpu_count() or 1
    oracle.build()
    shape = (L, L, L)
    P = oracle.Port(3)
    U, E = oracle.empty_fields(3, shape)
    P.random_links(shape, U, 0.3, 2)
    P.gaussian_efield(shape, E, np.sqrt(0.5), 1)
    kind = "port"
    runner = None
    if prefer_reference and oracle.ref_available(3):
        try:
            R = oracle.Ref(3)
            R.init(shape)
            R.set(U, E)
            runner = lambda n: R.leapfrog(dt, n)  # noqa: E731
            kind = "reference"
        except OSError:
            runner = None
    if runner is None:
        runner = lambda n: P.leapfrog(shape, U, E, dt, n)  # noqa: E731
    runner(1)  # warm-up (page-in, thread pool)
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps and (time.perf_counter() - t0) < min_seconds:
        runner(1)
        steps += 1
    el = time.perf_counter() - t0
    return {"value": 3 * L ** 3 * steps / el, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": f"{steps} leapfrog steps of the SU(3) {L}^3 lattice (FP64, OpenMP over z, "
                      f"{cores} threads), {el:.1f} s"}


# -------------------------------------------------------------- our arm
def run_ours(a):
    import torch
    import topologicalcymsolver_gb300 as tcym

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
    L, dt = a.size, a.dt
    V = L ** 3
    links = 3 * V
    ctx = tcym.Context(local)
    # clocks are sampled from the start of the initial-state preparation (seconds of FP64
    # restore work) through the timed region and the FP64 comparison: the timed region
    # itself (a few ms) is shorter than the sampling period
    clk = ClockSampler(local).__enter__()
    # initial state prepared in FP64 (Gauss restore to FP64 precision), then stored in FP32
    ic = tcym.Lattice(ctx, 3, (L, L, L), tcym.FP64)
    ic.random_links(0.3, 2 + 1000 * rank)
    ic.gaussian_efield(float(np.sqrt(0.5)), 1 + 1000 * rank)
    ic.gauss_restore(1e-12, 400)
    lat = tcym.Lattice(ctx, 3, (L, L, L), tcym.FP32)
    lat.copy_from(ic)
    lat.set_reunitarize_period(100)
    stream = torch.cuda.ExternalStream(lat.stream_handle(), device=torch.device("cuda", local))

    for _ in range(a.warmup):
        lat.leapfrog(dt, 1)
    lat.sync()
    steps_before = a.warmup

    # ---- timed region: K steps, per-launch events on the kernels' stream
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps + 1)]
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk.mark("timed_start")
    ev[0].record(stream)
    for k in range(a.steps):
        lat.leapfrog(dt, 1)
        ev[k + 1].record(stream)
    ev[-1].synchronize()
    torch.cuda.synchronize()
    clk.mark("timed_end")
    if ws > 1:
        torch.distributed.barrier()
    per = [ev[k].elapsed_time(ev[k + 1]) * 1e-3 for k in range(a.steps)]
    total = ev[0].elapsed_time(ev[-1]) * 1e-3
    reunits = sum(1 for s in range(steps_before + 1, steps_before + a.steps + 1) if s % 100 == 0)
    total = max_over_ranks(total, "cuda")
    value = ws * links * a.steps / total  # the units all ranks processed over the slowest rank's time

    # ---- the plain FP64 path (the compat header's default) on the same start, same K and W
    fp64 = None
    if not a.no_fp64:
        s64 = torch.cuda.ExternalStream(ic.stream_handle(), device=torch.device("cuda", local))
        for _ in range(a.warmup):
            ic.leapfrog(dt, 1)
        ic.sync()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(s64)
        for _ in range(a.steps):
            ic.leapfrog(dt, 1)
        f1.record(s64)
        f1.synchronize()
        t64 = f0.elapsed_time(f1) * 1e-3 / a.steps
        fp64 = {"value": links / t64, "unit": UNIT, "ms_per_step": t64 * 1e3, "steps": a.steps,
                "kernel": "k_step<SU3 FP64> (one site per thread, full 3x3 complex links, FP64 arithmetic)",
                "bytes_per_link_update": 416,
                "hbm_frac": round(416 * links / t64 / 1e9 / measured_peak()[0], 4),
                "fp32_over_fp64": round((total / a.steps) ** -1 / t64 ** -1, 2),
                "note": "plain FP64 device path (FP64 storage and arithmetic, no reunitarisation), same start, "
                        "same W and K as the headline; the accuracy of both over 1e4 steps is tested separately"}
    clk.__exit__()
    ic.close()

    # ---- end to end through the C ABI with pinned host buffers: the state lives in
    # host memory and every step moves it in and out (updated in place, a trajectory)
    Uh = torch.empty((V, 3, 18), dtype=torch.float64, pin_memory=True).numpy()
    Eh = torch.empty((V, 3, 8), dtype=torch.float64, pin_memory=True).numpy()
    lat.set_reunitarize_period(0)
    lat.download(Uh, Eh)
    n_e2e = max(1, a.e2e_steps)

    def timed(fn):
        fn()  # warm-up of the staging path
        if ws > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            fn()
        return ws * links * n_e2e / max_over_ranks(time.perf_counter() - t0, "cuda")

    def three_calls():
        lat.upload(Uh, Eh)
        lat.leapfrog(dt, 1)
        lat.download(Uh, Eh)

    e2e_seq = timed(three_calls)
    e2e_val = timed(lambda: lat.leapfrog_host(dt, Uh, Eh, Uh, Eh))
    e2e = {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(Uh.nbytes + Eh.nbytes),
           "d2h_bytes_per_step": int(Uh.nbytes + Eh.nbytes),
           "note": "per step: tcym_leapfrog_host on the AoS FP64 state in pinned host memory (upload, one leapfrog "
                   "step, download, pipelined over z-ordered chunks so both directions overlap), in place",
           "three_calls": {"value": e2e_seq, "note": "tcym_lattice_upload + tcym_leapfrog(1) + tcym_lattice_download"}}

    med = statistics.median(per)
    tile = "x".join(map(str, lat.tile())) if L % 2 == 0 else "per-site step (odd extent)"
    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_LINK * links / med / 1e9
    traffic = ncu_traffic()
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic,
            "kernel": ("k_step_pair<SU3 FP32> (site pairs in packed FP32; fused E and link update)" if L % 2 == 0
                       else "k_step<SU3 FP32> (fused E and link update)"),
            "bytes_per_link_update": BYTES_PER_LINK, "median_launch_ms": round(med * 1e3, 4),
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind}

    out = None
    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
               "ms_per_step": total / a.steps * 1e3, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(L, dt),
               "impl_config": impl_config(L, tile), "e2e": e2e, "roofline": roof, "clocks": clk.summary(),
               "gpu_launches": a.steps + reunits, "impl": "ours"}
        if fp64 is not None:
            out["fp64_path"] = fp64
        if ws == 1 and not a.no_cpu_baseline:
            cb = cpu_leapfrog_rate(L, dt, prefer_reference=False)
            out["cpu_baseline"] = cb
    lat.close()
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return out


def run_reference(a):
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    L, dt = a.size, a.dt
    # each bench step is one leapfrog step of the full lattice unless that would
    # take the run past a few minutes; then a smaller lattice is the sample
    import oracle
    oracle.build()

    def runner(Ls):
        shape = (Ls, Ls, Ls)
        P = oracle.Port(3)
        U, E = oracle.empty_fields(3, shape)
        P.random_links(shape, U, 0.3, 2)
        P.gaussian_efield(shape, E, np.sqrt(0.5), 1)
        if oracle.ref_available(3):  # the reference's own sources, where they were compiled on this host
            try:
                R = oracle.Ref(3)
                R.init(shape)
                R.set(U, E)
                return (lambda n: R.leapfrog(dt, n)), "reference"
            except OSError:
                pass
        return (lambda n: P.leapfrog(shape, U, E, dt, n)), "port"

    # one step of the full lattice sizes the sample: at most ~3 minutes in all
    run, kind = runner(L)
    t0 = time.perf_counter()
    run(1)
    per_step = time.perf_counter() - t0
    Ls = L
    while per_step * (a.steps + a.warmup) > 180.0 and Ls > 16:
        Ls //= 2
        per_step /= 8.0
    if Ls != L:
        run, kind = runner(Ls)
    run(a.warmup)
    t0 = time.perf_counter()
    run(a.steps)
    el = time.perf_counter() - t0
    value = 3 * Ls ** 3 * a.steps / el
    cores = os.cpu_count() or 1
    sample = (f"{a.steps} leapfrog steps of an SU(3) {Ls}^3 lattice after {a.warmup} warm-up steps, FP64, "
              f"OpenMP over z on {cores} threads" + ("" if Ls == L else f" (the {L}^3 lattice is the GPU workload; "
                                                                        "same per-link work)"))
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": el / a.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": config(L, dt), "impl": "reference",
            "impl_config": reference_impl_config(cores),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    a = parse()
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    if a.workload != "leapfrog":
        from topologicalcymsolver_gb300 import workloads
        out = workloads.run(a.workload, a) if dist_env()[1] == 0 else None
    elif a.impl == "reference":
        out = run_reference(a)
    else:
        out = run_ours(a)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
