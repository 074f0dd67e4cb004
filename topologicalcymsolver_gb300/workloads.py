"""Workload generators and runners for the batched configurations.

ensemble: 256 independent thermal leapfrog trajectories, each SU(2) or SU(3)
  (50/50), L uniform in {16, 24, 32, 48}, dt = 0.05, E-field variance T uniform
  in [0.3, 1.0], fields from the Philox stream of seed 5 + index, Gauss-restored
  in FP64 to 1e-10, stepped in FP32 storage with FP64 reductions, in batched
  graph-captured launches (tcym_ensemble_*).  Compared with the same lattices
  stepped by per-lattice launches and with the plain FP64 path.
serve: a Poisson request stream at 80% of the measured sustainable throughput (the
  steady-state rate of a server kept full by a closed loop of 48 requests in flight);
  each request: SU(2)/SU(3) 50/50, L uniform over {24, 32, 48, 64, 96, 128}
  (log-spaced, so uniform in log L), T uniform in [0.3, 1.0], leapfrog or
  Langevin (gamma = 1) 50/50, steps log-uniform in [1000, 20000], N_CS(t)
  every 20 steps (tcym_server_*).

Inputs are synthetic: seeded Philox fields with the configurations' distributions.
"""
from __future__ import annotations

import json
import math
import sys
import time

import numpy as np

from . import DYN_LANGEVIN, DYN_LEAPFROG, FP32, FP64, Context, Ensemble, Lattice, Server

GB = 1 << 30


def ensemble_specs(n: int = 256, seed: int = 5):
    """(nc, L, T, field seed) of each trajectory."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nc = 2 if rng.random() < 0.5 else 3
        L = int(rng.choice([16, 24, 32, 48]))
        T = float(rng.uniform(0.3, 1.0))
        out.append((nc, L, T, seed + i))
    return out


def thermal_lattice(ctx: Context, nc: int, L: int, T: float, seed: int, precision: int, tol: float = 1e-10):
    """U = 1, E ~ N(0, T) Gauss-restored in FP64, stored in `precision`."""
    ic = Lattice(ctx, nc, (L, L, L), FP64)
    ic.set_zero()
    ic.gaussian_efield(math.sqrt(T), seed)
    ic.gauss_restore(tol, 5000)
    if precision == FP64:
        return ic
    lat = Lattice(ctx, nc, (L, L, L), precision)
    lat.copy_from(ic)
    ic.close()
    return lat


def run_ensemble(a):
    ctx = Context(0)
    specs = ensemble_specs(a.trajectories)
    lats = [thermal_lattice(ctx, nc, L, T, s, FP32) for nc, L, T, s in specs]
    links = sum(3 * L ** 3 for _, L, _, _ in specs)
    dt = 0.05
    ens = Ensemble(ctx)
    for lat in lats:
        ens.add(lat, dt)
    chunk = 100
    ens.step(max(a.warmup, 3))
    steps = max(chunk, (a.steps // chunk) * chunk)
    t0 = time.perf_counter()
    for _ in range(steps // chunk):
        ens.step(chunk)
    t_ens = time.perf_counter() - t0
    rate = links * steps / t_ens
    # per-lattice launches, bounded samples
    nseq = 50
    t0 = time.perf_counter()
    for _ in range(nseq):
        for lat in lats:
            lat.leapfrog(dt, 1)
            lat.sync()
    seq_serial = links * nseq / (time.perf_counter() - t0)
    t0 = time.perf_counter()
    for _ in range(nseq):
        for lat in lats:
            lat.leapfrog(dt, 1)
    for lat in lats:
        lat.sync()
    seq_concurrent = links * nseq / (time.perf_counter() - t0)
    ens.close()
    for lat in lats:
        lat.close()
    # the plain FP64 path: the same trajectories in FP64 storage, batched
    lats64 = [thermal_lattice(ctx, nc, L, T, s, FP64) for nc, L, T, s in specs]
    e64 = Ensemble(ctx)
    for lat in lats64:
        e64.add(lat, dt)
    e64.step(3)
    n64 = 20
    t0 = time.perf_counter()
    e64.step(n64)
    fp64 = links * n64 / (time.perf_counter() - t0)
    e64.close()
    for lat in lats64:
        lat.close()
    ctx.close()
    n_su3 = sum(1 for s in specs if s[0] == 3)
    return {
        "metric": "ensemble trajectories/s (256 mixed SU(2)/SU(3) thermal trajectories, 2000 steps each)",
        "value": a.trajectories * (steps / 2000.0) / t_ens, "unit": "trajectories/s", "higher_is_better": True,
        "n_gpus": 1, "steps": steps, "warmup": max(a.warmup, 3), "dtype": "f32", "data": "synthetic",
        "vs_baseline": None, "impl": "ours",
        "config": {"workload": f"{a.trajectories} trajectories ({n_su3} SU(3)), L in {{16,24,32,48}}, dt=0.05, "
                               "T in [0.3,1], FP32 storage, FP64 reductions, graph chunks of 100 steps",
                   "link_updates_per_step": links},
        "link_updates_per_s": rate,
        "per_lattice_launches_serialized": seq_serial,
        "per_lattice_launches_concurrent_streams": seq_concurrent,
        "fp64_ensemble": fp64,
        "speedup_vs_serialized_launches": rate / seq_serial,
        "speedup_vs_concurrent_launches": rate / seq_concurrent,
        "speedup_vs_fp64": rate / fp64,
    }


def serve_requests(n: int, seed: int = 6):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        out.append(dict(nc=2 if rng.random() < 0.5 else 3, L=int(rng.choice([24, 32, 48, 64, 96, 128])),
                        T=float(rng.uniform(0.3, 1.0)),
                        dynamics=DYN_LANGEVIN if rng.random() < 0.5 else DYN_LEAPFROG,
                        nsteps=int(round(math.exp(rng.uniform(math.log(1000), math.log(20000))))),
                        seed=seed * 1000 + i))
    return out


def _work(r, stride=20):
    return 3 * r["L"] ** 3 * int(math.ceil(r["nsteps"] / stride) * stride)


def sustainable_rate(ctx, budget, dt, in_flight=48, warm_s=5.0, window_s=30.0, seed=60):
    """Aggregate link-updates/s of a server kept full: a closed loop holds `in_flight`
    requests from the request distribution queued or running, replacing each one as it
    finishes, and the server's link-update counter is read over `window_s` seconds after
    `warm_s` of ramp-up.  The server is closed afterwards (its requests abandoned)."""
    srv = Server(ctx, budget, max_active=512, stride=20)
    pool = serve_requests(100000, seed=seed)
    k, live = 0, []

    def top_up():
        nonlocal k
        while len(live) < in_flight:
            r = pool[k]
            k += 1
            live.append(srv.submit(nc=r["nc"], L=r["L"], T=r["T"], nsteps=r["nsteps"], dynamics=r["dynamics"],
                                   dt=dt[r["dynamics"]], gamma=1.0, precision=FP32, seed=r["seed"]))

    top_up()
    t0, mark = time.perf_counter(), None
    while True:
        live[:] = [i for i in live if srv.status(i)[0] in (0, 1)]
        top_up()
        now = time.perf_counter()
        if mark is None and now - t0 >= warm_s:
            mark = (now, srv.stats()["link_updates"])
        elif mark is not None and now - mark[0] >= window_s:
            rate = (srv.stats()["link_updates"] - mark[1]) / (now - mark[0])
            srv.close()
            return rate
        time.sleep(0.02)


def run_serve(a, progress=sys.stderr):
    ctx = Context(0)
    reqs = serve_requests(a.requests)
    dt = {DYN_LEAPFROG: 0.05, DYN_LANGEVIN: 0.02}
    budget = 200 * GB
    srv = Server(ctx, budget, max_active=512, stride=20)

    def submit(r):
        return srv.submit(nc=r["nc"], L=r["L"], T=r["T"], nsteps=r["nsteps"], dynamics=r["dynamics"],
                          dt=dt[r["dynamics"]], gamma=1.0, precision=FP32, seed=r["seed"])

    # sustainable throughput: the steady state of a server kept full (on its own server)
    sustainable = sustainable_rate(ctx, budget, dt, warm_s=20.0, window_s=getattr(a, "serve_window", 30.0))
    print(json.dumps({"sustainable_link_updates_per_s": sustainable}), file=progress, flush=True)
    # Poisson arrivals at 80% of it
    mean_work = sum(_work(r) for r in reqs) / len(reqs)
    lam = 0.8 * sustainable / mean_work
    rng = np.random.default_rng(66)
    arrivals = np.cumsum(rng.exponential(1.0 / lam, size=len(reqs)))
    start = time.perf_counter()
    ids = []
    for r, ta in zip(reqs, arrivals):
        delay = start + ta - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        ids.append(submit(r))
    lat_s, failed = [], 0
    for k, i in enumerate(ids):
        rc = srv.wait(i, 7200)
        series, latency, rc2 = srv.result(i)
        if rc != 0:
            failed += 1
        lat_s.append(latency)
        if progress is not None and (k + 1) % 100 == 0:  # progress on stderr, so a cut-off run leaves data
            st = srv.stats()
            print(json.dumps({"progress": k + 1, "elapsed_s": time.perf_counter() - start,
                              "p50_so_far_s": float(np.percentile(lat_s, 50)),
                              "p99_so_far_s": float(np.percentile(lat_s, 99)), "queued": st["queued"],
                              "active": st["active"], "link_updates": st["link_updates"],
                              "prep_seconds": st["prep_seconds"]}), file=progress, flush=True)
    makespan = time.perf_counter() - start
    stats = srv.stats()
    tick_ms, tick_prep = srv.ticks()
    log = srv.tick_log()
    srv.close()
    ctx.close()
    total = sum(_work(r) for r in reqs)
    return {
        "metric": "serving: aggregate link-updates/s under a Poisson request stream at 80% of sustainable throughput",
        "value": total / makespan, "unit": "link-updates/s", "higher_is_better": True, "n_gpus": 1,
        "dtype": "f32", "data": "synthetic", "vs_baseline": None, "impl": "ours",
        "config": {"workload": f"{len(reqs)} requests (Poisson, seed 6), SU(2)/SU(3), L in {{24..128}}, "
                               "T in [0.3,1], leapfrog dt 0.05 / Langevin dt 0.02 gamma 1, steps log-uniform "
                               "[1000, 20000], N_CS every 20 steps, FP32 storage, budget 200 GiB"},
        "p50_latency_s": float(np.percentile(lat_s, 50)), "p99_latency_s": float(np.percentile(lat_s, 99)),
        "requests": len(reqs), "failed": failed, "sustainable_link_updates_per_s": sustainable,
        "offered_requests_per_s": lam, "makespan_s": makespan, "server_link_updates": stats["link_updates"],
        "prep_seconds": stats["prep_seconds"], "ticks": stats["ticks"],
        "tick_ms": {"median": float(np.median(tick_ms)) if len(tick_ms) else None,
                    "median_while_preparing": (float(np.median(tick_ms[tick_prep > 0]))
                                               if np.any(tick_prep > 0) else None),
                    "median_idle_preparers": (float(np.median(tick_ms[tick_prep == 0]))
                                              if np.any(tick_prep == 0) else None),
                    "note": "last <= 8192 ticks; a tick = stride steps of every running request + its N_CS sample"},
        "tick_log": _tick_summary(log),
    }


def _tick_summary(log):
    """Where the request loop's time went over the recorded ticks: the link-update rate
    inside ticks, the share of wall time in ticks and between them, by preparations
    under way and by running requests."""
    if len(log) == 0:
        return None
    ms, gap, lu = log["ms"], log["gap_ms"], log["link_updates"]
    busy = log["preparing"] > 0
    wall = float(ms.sum() + gap.sum())
    out = {"ticks": int(len(log)), "wall_s": wall * 1e-3,
           "in_tick_link_updates_per_s": float(lu.sum() / ms.sum() * 1e3),
           "share_in_ticks": float(ms.sum() / wall), "gap_ms_median": float(np.median(gap)),
           "gap_ms_total_s": float(gap.sum() * 1e-3), "active_median": float(np.median(log["active"]))}
    for name, sel in (("while_preparing", busy), ("preparers_idle", ~busy)):
        if np.any(sel):
            out[f"in_tick_link_updates_per_s_{name}"] = float(lu[sel].sum() / ms[sel].sum() * 1e3)
            out[f"ticks_{name}"] = int(sel.sum())
    return out


def run(name: str, a):
    if name == "ensemble":
        return run_ensemble(a)
    if name == "serve":
        return run_serve(a)
    raise ValueError(name)
