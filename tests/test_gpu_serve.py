"""The continuous-batching request loop (tcym_server_*).

* a request's N_CS series is bit-identical alone and inside a mix of other
  requests arriving before and after it;
* it equals the series of the same trajectory stepped through the lattice API;
* admission keeps the device-memory budget, admits waiting requests as others
  finish, and refuses a request that can never fit;
* failures are handled on the host: a bounded wait times out, and a request
  whose initial fields are NaN (fault injected through its parameters) fails
  alone while the others complete;
* a request's preparation (initial fields and their Gauss restore in the
  request's precision) runs on its own threads and streams: the running requests
  keep ticking meanwhile;
* a served request's N_CS series equals the oracle's run of the same trajectory.
"""
import time

import numpy as np
import pytest

import oracle
import topologicalcymsolver_gb300 as tcym

pytestmark = pytest.mark.gpu

GB = 1 << 30


def test_series_alone_equals_series_in_mix(ctx):
    probe = dict(nc=3, L=6, T=0.6, nsteps=100, dynamics=tcym.DYN_LANGEVIN, dt=0.02, gamma=1.0, seed=77)
    a = tcym.Server(ctx, 4 * GB, stride=20)
    rid = a.submit(**probe)
    assert a.wait(rid, 300) == 0
    alone, _, rc = a.result(rid)
    assert rc == 0 and alone.shape == (5, 2)
    a.close()
    b = tcym.Server(ctx, 4 * GB, stride=20)
    rng = np.random.default_rng(1)
    others = []
    for i in range(6):
        others.append(b.submit(nc=int(rng.choice([2, 3])), L=int(rng.choice([4, 5, 8])), T=float(rng.uniform(0.3, 1)),
                               nsteps=int(rng.choice([40, 120, 200])), dynamics=int(rng.integers(0, 2)), seed=i))
    rid = b.submit(**probe)
    for i in range(6, 10):
        others.append(b.submit(nc=2, L=6, T=0.5, nsteps=60, seed=i))
    assert b.wait(rid, 300) == 0
    mixed, _, rc = b.result(rid)
    assert rc == 0
    assert np.array_equal(alone, mixed)
    for o in others:
        assert b.wait(o, 300) == 0
    b.close()


def test_series_equals_lattice_path(ctx):
    nc, L, T, n, stride = 2, 8, 0.7, 60, 20
    s = tcym.Server(ctx, 2 * GB, stride=stride)
    rid = s.submit(nc=nc, L=L, T=T, nsteps=n, dynamics=tcym.DYN_LEAPFROG, dt=0.05, precision=tcym.FP64, seed=5)
    assert s.wait(rid, 300) == 0
    series, latency, _ = s.result(rid)
    s.close()
    lat = tcym.Lattice(ctx, nc, (L, L, L), tcym.FP64)
    lat.set_zero()
    lat.gaussian_efield(np.sqrt(T), 5)
    lat.gauss_restore(1e-12, 400)
    lat.ncs_track(stride)
    lat.ncs_reset()
    ref = []
    for k in range(n // stride):
        lat.leapfrog(0.05, stride)
        ref.append(lat.ncs())
    assert np.allclose(series[:, 0], [stride * (k + 1) for k in range(n // stride)])
    assert np.allclose(series[:, 1], ref, rtol=1e-9, atol=1e-12)
    assert latency > 0


@pytest.mark.parametrize("prec", [tcym.FP64, tcym.FP32], ids=["fp64", "fp32"])
def test_served_request_against_oracle(ctx, oracle_port, prec):
    """An SU(3) 6^3 leapfrog request served beside two others, against the oracle run of
    the same trajectory: U = 1, E ~ N(0, T) from the request's Philox stream, Gauss
    restored as the server restores (FP64: 1e-12, FP32: 1e-6, at most 400 iterations),
    then strides of 20 steps with N_CS += dt * 20 * (clover E.B) / 8 pi^2 after each.
    FP64 within 1e-9 of the series' scale, FP32 within 1e-5."""
    nc, L, T, n, stride, dt, seed = 3, 6, 0.7, 60, 20, 0.05, 41
    s = tcym.Server(ctx, 2 * GB, stride=stride)
    others = [s.submit(nc=2, L=8, T=0.5, nsteps=100, seed=1), s.submit(nc=3, L=4, T=0.9, nsteps=40, seed=2)]
    rid = s.submit(nc=nc, L=L, T=T, nsteps=n, dynamics=tcym.DYN_LEAPFROG, dt=dt, precision=prec, seed=seed)
    assert s.wait(rid, 300) == 0
    series, _, rc = s.result(rid)
    for o in others:
        assert s.wait(o, 300) == 0
    s.close()
    P = oracle_port[nc]
    shape = (L, L, L)
    U, E = oracle.empty_fields(nc, shape)
    P.set_zero(shape, U, E)
    P.gaussian_efield(shape, E, np.sqrt(T), seed)
    P.gauss_restore(shape, U, E, 1e-12 if prec == tcym.FP64 else 1e-6, 400)
    ref, total = [], 0.0
    for _ in range(n // stride):
        P.leapfrog(shape, U, E, dt, stride)
        total += dt * stride * P.edotb_clover(shape, U, E) / (8 * np.pi ** 2)
        ref.append(total)
    ref = np.array(ref)
    scale = max(np.abs(ref).max(), 1e-3)
    err = np.abs(series[:, 1] - ref).max() / scale
    print(f"\nmeasured served request SU(3) 6^3 prec={prec} vs oracle: N_CS {err:.2e} of {scale:.3e}")
    assert rc == 0 and np.allclose(series[:, 0], [stride * (k + 1) for k in range(n // stride)])
    assert err < (1e-9 if prec == tcym.FP64 else 1e-5)


def test_admission_by_memory_budget(ctx):
    # one SU(3) 16^3 FP32 request needs ~6.8 MB: a 16 MB budget holds two at a time
    s = tcym.Server(ctx, 16 << 20, stride=10)
    ids = [s.submit(nc=3, L=16, T=0.5, nsteps=30, seed=i) for i in range(6)]
    peak = 0
    for rid in ids:
        while s.wait(rid, 0.01) == 5:
            peak = max(peak, s.stats()["bytes_in_use"])
    assert peak <= 16 << 20
    assert all(s.result(rid)[2] == 0 for rid in ids)
    st = s.stats()
    assert st["completed"] == 6 and st["failed"] == 0 and st["bytes_in_use"] == 0
    with pytest.raises(tcym.TcymError) as ei:
        s.submit(nc=3, L=64, T=0.5, nsteps=10)
    assert ei.value.code == 6
    s.close()


def test_bounded_wait_and_injected_fault(ctx):
    s = tcym.Server(ctx, 4 * GB, stride=20)
    slow = s.submit(nc=3, L=24, T=0.5, nsteps=4000, seed=1)
    assert s.wait(slow, 0.0) == 5  # bounded wait runs out: TCYM_ERR_TIMEOUT
    bad = s.submit(nc=2, L=6, T=float("nan"), nsteps=40, seed=2)
    good = s.submit(nc=2, L=6, T=0.5, nsteps=40, seed=3)
    assert s.wait(bad, 300) == 4  # non-finite initial state: the request fails alone
    assert s.wait(good, 300) == 0
    st = s.stats()
    assert st["failed"] == 1
    s.close()  # abandons the slow request


def test_ticks_continue_while_a_large_request_is_prepared(ctx):
    """Eight small requests tick; a 128^3 SU(3) FP64 request arrives, whose preparation
    (Gaussian fields, Gauss restore to 1e-12 in FP64) takes far longer than a tick.  The
    ticks during that preparation stay close to the ticks before it (measured: 0.3 ms
    before, 0.84-0.95 ms median during a 7 s preparation): the loop does not stop for
    an admission."""
    s = tcym.Server(ctx, 64 * GB, stride=20)
    small = [s.submit(nc=2, L=24, T=0.5, nsteps=400000, seed=i) for i in range(8)]
    t0 = time.time()
    while s.stats()["active"] < 8 and time.time() - t0 < 60:
        time.sleep(0.01)
    time.sleep(0.5)
    ms, _ = s.ticks()
    base = float(np.median(ms[-100:]))
    big = s.submit(nc=3, L=128, T=0.6, nsteps=20, precision=tcym.FP64, seed=99)
    assert s.wait(big, 300) == 0
    ms, prep = s.ticks()
    during = ms[prep > 0]
    st = s.stats()
    print(f"\nmeasured serve ticks: base median {base:.3f} ms, during preparation median "
          f"{np.median(during):.3f} ms max {during.max():.3f} ms over {len(during)} ticks; "
          f"preparation {st['prep_seconds']:.3f} s")
    assert len(during) >= 5
    assert np.median(during) < 4.0 * base + 1.0
    assert during.max() < 0.5 * 1e3 * st["prep_seconds"]  # no tick waited for the whole preparation
    # the full records: each tick's work and the time between ticks
    log = s.tick_log()
    assert len(log) > 0 and np.all(log["ms"] > 0)
    assert np.all(log["active"] >= 1) and np.all(log["gap_ms"] >= 0)
    small_work = 3 * 16 ** 3 * 20  # one 16^3 request's stride of 20 steps
    assert np.all(log["link_updates"] >= small_work)
    for rid in small:
        assert s.status(rid)[0] == tcym.REQ_RUNNING
    s.close()  # abandons the small requests
