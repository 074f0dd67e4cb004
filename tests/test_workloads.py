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
