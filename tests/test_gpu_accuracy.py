"""Accuracy of each observable against the FP64 oracle, and ensemble statistics.

* Per observable (T00, E^2, B^2, Gauss max/rms, unitarity max, clover and improved
  E.B, Kahan N_CS), the relative error of the FP64 and FP32 device paths against
  the oracle over the first 100 steps of an SU(2) 16^3 leapfrog start and of an
  SU(3) Langevin start (32^3 here); the table is printed
  (pytest -s) and bounded: FP64 1e-10, FP32 1e-5 (E.B and N_CS: relative to the
  mean |E.B|, since they are sums that cancel).
* N_CS diffusion: 24 thermal SU(2) 12^3 trajectories stepped 2000 steps in an
  ensemble in FP32 and in FP64 from identical starts; chaos decorrelates the
  trajectories, so only the ensemble means of (Delta N_CS)^2 must agree, within
  three standard errors, and the Gauss-law and unitarity violations stay bounded.
"""
import numpy as np
import pytest

import oracle
import topologicalcymsolver_gb300 as tcym

pytestmark = pytest.mark.gpu


def _series(lat, P, shape, U, E, step, n, every):
    got, ref = [], []
    for _ in range(n // every):
        step(lat, P, U, E, every)
        o = lat.observables()
        r = P.observables(shape, U, E)
        got.append([o.T00, o.electric, o.magnetic, o.gauss_absmax, o.gauss_rms, o.unit_max, o.edotb,
                    lat.edotb_improved(), lat.ncs()])
        ref.append([r[0], r[1], r[2], r[15], r[10], r[11], r[13], P.edotb_improved(shape, U, E), 0.0])
    return np.array(got), np.array(ref)


NAMES = ["T00", "E^2/2", "B^2/2", "Gauss |max|", "Gauss rms", "unitarity max", "clover E.B", "improved E.B",
         "N_CS"]


@pytest.mark.parametrize("prec", [tcym.FP64, tcym.FP32], ids=["fp64", "fp32"])
@pytest.mark.parametrize("start", ["su2_leapfrog", "su3_langevin"])
def test_observable_errors(ctx, oracle_port, start, prec):
    if start == "su2_leapfrog":
        nc, shape, P = 2, (16, 16, 16), oracle_port[2]
        U, E = oracle.empty_fields(2, shape)
        P.set_zero(shape, U, E)
        P.gaussian_efield(shape, E, np.sqrt(0.5), 1)
        P.gauss_restore(shape, U, E, 1e-14, 10000)

        def step(lat, P, U, E, n):
            lat.leapfrog(0.05, n)
            P.leapfrog(shape, U, E, 0.05, n)
        dt = 0.05
    else:
        nc, shape, P = 3, (32, 32, 32), oracle_port[3]
        U, E = oracle.empty_fields(3, shape)
        P.random_links(shape, U, 0.3, 2)
        k = [0]

        def step(lat, P, U, E, n):
            lat.langevin(0.02, 1.0, 0.6, 3, k[0], n)
            P.langevin(shape, U, E, 0.02, 1.0, 0.6, 3, k[0], n)
            k[0] += n
        dt = 0.02
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.set_reunitarize_period(0)
    lat.upload(U, E)
    if prec == tcym.FP32:
        U, E = lat.download()
    lat.ncs_track(10)
    lat.ncs_reset()
    got, ref = _series(lat, P, shape, U, E, step, 100, 10)
    # the oracle's Kahan-free N_CS at the same sampling: dt * every * clover E.B / (8 pi^2), summed
    ref[:, 8] = np.cumsum(ref[:, 6]) * dt * 10 / (8 * np.pi ** 2)
    scale = np.abs(ref).max(axis=0)
    scale[6:9] = np.maximum(np.abs(ref[:, 6:8]).mean(), 1e-12)  # sums that cancel: relative to mean |E.B|
    scale[8] = max(np.abs(ref[:, 6]).mean() * dt * 10 / (8 * np.pi ** 2) * len(ref), 1e-12)
    err = np.abs(got - ref).max(axis=0) / np.maximum(scale, 1e-300)
    tol = 1e-10 if prec == tcym.FP64 else 1e-5
    print(f"\n{start} {'FP64' if prec == tcym.FP64 else 'FP32'} max relative error over 100 steps:")
    for name, e in zip(NAMES, err):
        print(f"  {name:14s} {e:.2e}")
    for i, name in enumerate(NAMES):
        if name == "unitarity max" or (start == "su2_leapfrog" and name.startswith("Gauss")):
            # violations of a restored / unitary state are rounding-level absolute numbers
            # (~1e-14 in FP64, ~1e-7 in FP32): bounded absolutely
            assert np.abs(got[:, i]).max() < (1e-10 if prec == tcym.FP64 else 1e-4), name
        else:  # the Langevin noise breaks Gauss's law (the SU(3) Langevin run): its violation compares relatively
            assert err[i] < tol, (name, err[i])


def test_ncs_diffusion_fp32_vs_fp64(ctx):
    n, L, steps = 24, 12, 2000
    rng = np.random.default_rng(17)
    Ts = rng.uniform(0.4, 0.8, size=n)
    lats = {tcym.FP64: [], tcym.FP32: []}
    for i in range(n):
        ic = tcym.Lattice(ctx, 2, (L, L, L), tcym.FP64)
        ic.set_zero()
        ic.gaussian_efield(np.sqrt(Ts[i]), 100 + i)
        ic.gauss_restore(1e-12, 5000)
        lats[tcym.FP64].append(ic)
        l32 = tcym.Lattice(ctx, 2, (L, L, L), tcym.FP32)
        l32.copy_from(ic)
        lats[tcym.FP32].append(l32)
    d2 = {}
    for prec, ls in lats.items():
        ens = tcym.Ensemble(ctx)
        for lat in ls:
            ens.add(lat, 0.05)
        ncs = np.zeros(n)  # new lattices start their Kahan N_CS at 0
        for _ in range(steps // 20):
            ens.step(20)
            _, ncs = ens.measure(20)  # N_CS += 20 dt E.B / (8 pi^2) per member
        d2[prec] = ncs ** 2
        for lat in ls:
            o = lat.observables()
            assert o.gauss_absmax < (1e-9 if prec == tcym.FP64 else 1e-3)
            assert o.unit_max < (1e-12 if prec == tcym.FP64 else 1e-5)
        ens.close()
    m64, m32 = d2[tcym.FP64].mean(), d2[tcym.FP32].mean()
    se = np.sqrt(d2[tcym.FP64].var(ddof=1) / n + d2[tcym.FP32].var(ddof=1) / n)
    print(f"\n<dN_CS^2> over {steps} steps: FP64 {m64:.4e}, FP32 {m32:.4e}, standard error {se:.2e}")
    assert abs(m32 - m64) < 3 * se + 1e-12
