"""The synthetic workloads of bench.py on the CPU: the ensemble's and the request
stream's distributions are the configurations' (256 mixed trajectories; Poisson
requests with L log-uniform over {24..128} and steps log-uniform in [1000, 20000]),
and seeded, so every run measures the same work."""
import math

import numpy as np

from topologicalcymsolver_gb300 import workloads


def test_ensemble_specs_are_the_bench_workload():
    specs = workloads.ensemble_specs(256)
    assert specs == workloads.ensemble_specs(256)  # seeded
    assert {L for _, L, _, _ in specs} == {16, 24, 32, 48}
    assert all(0.3 <= T <= 1.0 for _, _, T, _ in specs)
    assert len({s for _, _, _, s in specs}) == 256
    n_su3 = sum(1 for nc, _, _, _ in specs if nc == 3)
    assert n_su3 == 119  # the bench line's "256 trajectories (119 SU(3))"
    assert sum(3 * L ** 3 for _, L, _, _ in specs) == 30005760  # its link_updates_per_step


def test_request_stream_distribution():
    reqs = workloads.serve_requests(2000)
    assert reqs == workloads.serve_requests(2000)
    su3 = np.mean([r["nc"] == 3 for r in reqs])
    langevin = np.mean([r["dynamics"] == workloads.DYN_LANGEVIN for r in reqs])
    assert abs(su3 - 0.5) < 0.05 and abs(langevin - 0.5) < 0.05
    Ls = [r["L"] for r in reqs]
    assert set(Ls) == {24, 32, 48, 64, 96, 128}
    steps = np.array([r["nsteps"] for r in reqs])
    assert steps.min() >= 1000 and steps.max() <= 20000
    # log-uniform: the median near the geometric mean of the bounds, log(steps) flat
    assert abs(np.median(steps) / math.sqrt(1000 * 20000) - 1) < 0.1
    h, _ = np.histogram(np.log(steps), bins=5)
    assert h.min() > 0.7 * h.mean()
    assert len({r["seed"] for r in reqs}) == 2000


def test_tick_summary_splits_time_and_rates():
    """The serve workload's summary of the server's tick log: the link-update rate inside
    ticks, the share of wall time inside them, and both split by whether a preparation
    was under way, from records laid out as tcym_tick."""
    import numpy as np

    import topologicalcymsolver_gb300 as tcym
    from topologicalcymsolver_gb300 import workloads

    log = np.zeros(4, dtype=tcym.TICK_DTYPE)
    log["ms"] = [100.0, 100.0, 200.0, 100.0]
    log["gap_ms"] = [0.0, 10.0, 10.0, 80.0]
    log["link_updates"] = [1e9, 1e9, 1e9, 2e9]
    log["active"] = [3, 3, 4, 5]
    log["preparing"] = [0, 1, 1, 0]
    s = workloads._tick_summary(log)
    assert s["ticks"] == 4 and abs(s["wall_s"] - 0.6) < 1e-12
    assert abs(s["share_in_ticks"] - 500.0 / 600.0) < 1e-12
    assert abs(s["in_tick_link_updates_per_s"] - 5e9 / 0.5) < 1e-3
    assert abs(s["in_tick_link_updates_per_s_while_preparing"] - 2e9 / 0.3) < 1e-3
    assert abs(s["in_tick_link_updates_per_s_preparers_idle"] - 3e9 / 0.2) < 1e-3
    assert s["ticks_while_preparing"] == 2 and s["ticks_preparers_idle"] == 2
    assert abs(s["gap_ms_total_s"] - 0.1) < 1e-12 and s["active_median"] == 3.5
    assert workloads._tick_summary(log[:0]) is None
