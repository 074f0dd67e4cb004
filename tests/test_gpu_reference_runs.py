"""The reference runs this path is measured on, as parity tests (GPU through the C ABI).

SU(2) 16^3 leapfrog: U = 1, E ~ N(0, 1/2) (seed 1) Gauss-restored, 1000 leapfrog
  steps at dt 0.05, observables every 10 steps: compared with the reference's own
  series (tests/golden/ref_leapfrog_su2_16.npz) pointwise over the first 100 steps
  and, beyond the chaotic horizon, through the conserved energy.
SU(3) 64^3 Langevin: dt 0.02, gamma 1, T 0.6, links exp(i theta lambda/2)
  theta ~ N(0, 0.09) (seed 2), E = 0, noise seed 3: pointwise against the FP64
  oracle fed the identical noise for 100 steps (FP64 <= 1e-10, FP32 <= 1e-5
  relative), and the Kahan-integrated N_CS over the first 10.
SU(2) 96^3 cooling: leapfrog, then gradient-flow cooling sweeps at dtau 0.02:
  at 32^3 against the oracle's checkerboard restatement every 10 sweeps; at the
  full 96^3 (2000 leapfrog steps, 500 sweeps) the FP32 checkerboard series
  against the oracle's and the FP64 simultaneous series against the reference's
  own (tests/golden/ref_cooling_su2_96.npz).
energy: over 10^4 leapfrog steps neither path's mean energy drifts and the
  FP32 path's stays with the FP64 path's.
"""
import os

import numpy as np
import pytest

import oracle
import topologicalcymsolver_gb300 as tcym

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


# tolerances: energies relative; E.B (a sum that cancels) relative to its mean magnitude over
# the compared records, FP32 10x the measured 2.0e-6
@pytest.mark.parametrize("prec,tol_e,tol_edb", [(tcym.FP64, 1e-10, 1e-10), (tcym.FP32, 1e-5, 2e-5)])
def test_su2_16_leapfrog_against_reference_series(ctx, prec, tol_e, tol_edb):
    d = dict(np.load(os.path.join(G, "ref_leapfrog_su2_16.npz")))
    s = d["series"]
    shape = (16, 16, 16)
    ic = tcym.Lattice(ctx, 2, shape, tcym.FP64)
    ic.set_zero()
    ic.gaussian_efield(1.0 / np.sqrt(2.0), 1)
    ic.gauss_restore(1e-14, 10000)
    assert rel(ic.download()[1], d["E_ic"]) < 1e-12
    lat = ic
    if prec == tcym.FP32:
        lat = tcym.Lattice(ctx, 2, shape, prec)
        lat.copy_from(ic)
    T00 = []
    edb_scale = np.abs(s[:11, 13]).mean()
    err_e = err_edb = 0.0
    for rec in range(len(s)):
        if rec:
            lat.leapfrog(float(d["dt"]), int(d["every"]))
        o = lat.observables()
        v = o.as_oracle_vector()
        T00.append(v[0])
        if rec <= 10:  # the first 100 steps: pointwise
            for k in (0, 1, 2):
                if s[rec][k] != 0.0:  # the magnetic energy of the unit-link start is exactly 0
                    err_e = max(err_e, abs(v[k] - s[rec][k]) / abs(s[rec][k]))
                assert abs(v[k] - s[rec][k]) <= tol_e * abs(s[rec][k]) + 1e-15, (rec, k, v[k], s[rec][k])
            err_edb = max(err_edb, abs(v[13] - s[rec][13]) / edb_scale)
            assert abs(v[13] - s[rec][13]) <= tol_edb * edb_scale, (rec, v[13], s[rec][13])
        assert o.gauss_absmax < (1e-11 if prec == tcym.FP64 else 1e-4)
        assert o.unit_max < (1e-12 if prec == tcym.FP64 else 1e-5)
    print(f"\nmeasured SU(2) 16^3 series prec={prec}: energies {err_e:.2e}, E.B / mean |E.B| {err_edb:.2e}")
    T00, Tref = np.array(T00), s[:, 0]
    # beyond the chaotic horizon both conserve the energy: they agree to the leapfrog fluctuation
    assert np.abs(T00[20:] - Tref[20:]).max() < 5e-3 * Tref.mean()
    assert abs(T00[-50:].mean() - Tref[-50:].mean()) < 1e-3 * Tref.mean()


@pytest.mark.parametrize("prec,tol", [(tcym.FP64, 1e-10), (tcym.FP32, 1e-5)])
def test_su3_64_langevin_identical_noise(ctx, oracle_port, prec, tol):
    P = oracle_port[3]
    shape = (64, 64, 64)
    U, E = oracle.empty_fields(3, shape)
    P.random_links(shape, U, 0.3, 2)
    lat = tcym.Lattice(ctx, 3, shape, prec)
    lat.random_links(0.3, 2)
    lat.set_reunitarize_period(0)
    Ug, _ = lat.download()
    assert rel(Ug, U) < (1e-13 if prec == tcym.FP64 else 5e-7)
    if prec == tcym.FP32:  # the oracle starts from the same rounded links
        U = Ug
    lat.upload(U, E)
    lat.ncs_track(1)
    lat.ncs_reset()
    dt, ncs, scale = 0.02, 0.0, 0.0
    for k in range(10):
        lat.langevin(dt, 1.0, 0.6, 3, k, 1)
        P.langevin(shape, U, E, dt, 1.0, 0.6, 3, k, 1)
        edb = P.edotb_clover(shape, U, E)
        ncs += dt * edb / (8 * np.pi ** 2)
        scale += dt * abs(edb) / (8 * np.pi ** 2)
    assert abs(lat.ncs() - ncs) <= 100 * tol * scale + 1e-13, (lat.ncs(), ncs, scale)
    lat.langevin(dt, 1.0, 0.6, 3, 10, 90)
    P.langevin(shape, U, E, dt, 1.0, 0.6, 3, 10, 90)
    Ug, Eg = lat.download()
    assert rel(Ug, U) < tol and rel(Eg, E) < tol, (rel(Ug, U), rel(Eg, E))


def _cooling_input(ctx, shape, nlf, tol=1e-14):
    lat = tcym.Lattice(ctx, 2, shape, tcym.FP64)
    lat.set_zero()
    lat.gaussian_efield(np.sqrt(0.5), 4)
    lat.gauss_restore(tol, 10000)
    lat.leapfrog(0.05, nlf)
    return lat


# links relative; the magnetic energy, which cooling drives down (so its relative error
# grows), FP32 to 5e-5 (6x the measured 8.3e-6)
@pytest.mark.parametrize("prec,tol,tol_mag", [(tcym.FP64, 1e-10, 1e-9), (tcym.FP32, 1e-5, 5e-5)])
def test_su2_cooling_sweeps_against_oracle(ctx, oracle_port, prec, tol, tol_mag):
    P = oracle_port[2]
    shape = (32, 32, 32)
    src = _cooling_input(ctx, shape, 200)
    U, E = src.download()
    lat = tcym.Lattice(ctx, 2, shape, prec)
    lat.copy_from(src)
    if prec == tcym.FP32:
        U, E = lat.download()
    mags = []
    for sweep in range(5):
        lat.flow(0.02, 10, tcym.FLOW_CHECKERBOARD)
        P.flow_checkerboard(shape, U, 0.02, 10)
        Ug, _ = lat.download()
        assert rel(Ug, U) < tol, (sweep, rel(Ug, U))
        o = lat.observables().as_oracle_vector()
        r = P.observables(shape, U, E)
        assert abs(o[2] - r[2]) <= tol_mag * r[2]
        mags.append(o[2])
    assert all(b < a for a, b in zip(mags, mags[1:]))  # cooling lowers the magnetic energy


def _cool_series(lat, mode, records):
    """`records` x 10 sweeps of dtau 0.02 in `mode`: (T00, ELECTRIC, MAGNETIC, cooled N_CS so far)
    after each 10."""
    out, t = [], 0.0
    for _ in range(records):
        t += lat.flow(0.02, 10, mode, calibrate=tcym.NCS_IMPROVED)
        o = lat.observables()
        out.append([o.T00, o.electric, o.magnetic, t])
    return np.array(out)


def _series_errors(got, ref):
    """Per record: |magnetic / reference - 1| and |N_CS - reference| over the reference's
    largest 10-sweep N_CS increment."""
    mag = np.abs(got[:, 2] / ref[:, 2] - 1)
    scale = np.abs(np.diff(np.concatenate([[0.0], ref[:, 3]]))).max()
    return mag, np.abs(got[:, 3] - ref[:, 3]) / scale


def test_su2_96_cooling_against_reference_run(ctx):
    """The SU(2) 96^3 cooling run at full size against tests/golden/ref_cooling_su2_96.npz:
    U = 1, E ~ N(0, 1/2) (seed 4) restored as the reference restores (1e-14, at most
    10000 iterations), 2000 leapfrog steps in FP64 (the start matches the reference's
    own, sampled at 64 sites and through its observables), then 500 sweeps of dtau 0.02
    with energy and cooled N_CS (improved E.B, trapezoid along the flow) every 10 sweeps,
    each flow in FP64 and in FP32 storage: checkerboard sweeps against the oracle's
    checkerboard series, simultaneous sweeps against the reference's own CalibrationUpdate
    series."""
    d = dict(np.load(os.path.join(G, "ref_cooling_su2_96.npz")))
    shape = (96, 96, 96)
    l64 = tcym.Lattice(ctx, 2, shape, tcym.FP64)
    l64.set_zero()
    l64.gaussian_efield(np.sqrt(0.5), 4)
    l64.gauss_restore(1e-14, 10000)
    l64.leapfrog(0.05, 2000)
    U, E = l64.download()
    idx = d["fp_sites"]
    fp_u, fp_e = rel(U[idx], d["fp_U"]), rel(E[idx], d["fp_E"])
    o = l64.observables().as_oracle_vector()
    fp_t = abs(o[0] / d["start_obs"][0] - 1)
    print(f"\nmeasured SU(2) 96^3 cooling start: U {fp_u:.2e} E {fp_e:.2e} T00 {fp_t:.2e}")
    assert fp_u < 1e-9 and fp_e < 1e-9 and fp_t < 1e-10
    n = len(d["checkerboard"])
    runs = {}
    for prec in (tcym.FP64, tcym.FP32):
        for mode, key in ((tcym.FLOW_CHECKERBOARD, "checkerboard"), (tcym.FLOW_SIMULTANEOUS, "simultaneous")):
            lat = tcym.Lattice(ctx, 2, shape, prec)
            lat.copy_from(l64)
            got = _cool_series(lat, mode, n)
            unit = lat.observables().unit_max
            lat.close()
            mag, ncs = _series_errors(got, d[key])
            name = f"{'FP64' if prec == tcym.FP64 else 'FP32'} {key}"
            runs[name] = (got, mag, ncs)
            print(f"measured SU(2) 96^3 cooling {name}: magnetic {mag[:3].max():.2e} (30 sweeps) "
                  f"{mag.max():.2e} (500), N_CS {ncs[:3].max():.2e} / {ncs.max():.2e}; unitarity {unit:.1e}")
            print("  magnetic per record " + " ".join(f"{x:.1e}" for x in mag))
            print("  N_CS per record     " + " ".join(f"{x:.1e}" for x in ncs))
    for name, (got, mag, ncs) in runs.items():
        assert np.all(np.diff(got[:, 2]) < 0), name  # cooling lowers B^2
        if name.startswith("FP64"):
            assert mag.max() < 1e-6 and ncs.max() < 1e-6, name
        else:
            # FP32 storage: the cooled field's magnetic energy (12 (1 - Re tr U_p / 2) a
            # site) falls 280-fold over the 500 sweeps to 4e-4 a site, and follows the
            # links' norms to first order; the increment-form exponentials and the FP64
            # reunitarisation every 10 sweeps keep them (measured: magnetic 6.5e-8 over
            # 30 sweeps, 3.3e-6 over 500; N_CS 2.9e-6)
            assert mag[:3].max() < 1e-6 and ncs[:3].max() < 1e-5, name
            assert mag.max() < 5e-5 and ncs.max() < 5e-5, name


def test_energy_drift_fp32_vs_fp64(ctx):
    shape = (32, 32, 32)
    l64 = tcym.Lattice(ctx, 3, shape, tcym.FP64)
    l64.set_zero()
    l64.gaussian_efield(np.sqrt(0.5), 11)
    l64.gauss_restore(1e-12, 4000)
    l64.leapfrog(0.05, 400)  # past the initial transient of B = 0
    l32 = tcym.Lattice(ctx, 3, shape, tcym.FP32)
    l32.copy_from(l64)
    e = {tcym.FP64: [], tcym.FP32: []}
    for _ in range(200):
        for lat, key in ((l64, tcym.FP64), (l32, tcym.FP32)):
            lat.leapfrog(0.05, 50)
            e[key].append(lat.observables().T00)
    e64, e32 = np.array(e[tcym.FP64]), np.array(e[tcym.FP32])
    # 10^4 steps: the mean energy does not drift between halves, in either precision,
    # and the FP32 path's mean stays with the FP64 path's (the bounds are a few
    # standard errors of the leapfrog fluctuation's mean at this volume)
    for x in (e64, e32):
        assert abs(x[100:].mean() - x[:100].mean()) / x.mean() < 2e-4
    assert abs(e32.mean() - e64.mean()) / e64.mean() < 2e-4
    assert l32.observables().unit_max < 1e-5  # periodic FP64 reunitarisation keeps FP32 links on the group


# relative to the largest increment of the series (it cancels): FP32 10x the measured 4.0e-7
@pytest.mark.parametrize("prec,tol", [(tcym.FP64, 1e-9), (tcym.FP32, 4e-6)])
def test_su2_cooled_ncs_series(ctx, oracle_port, prec, tol):
    """The cooling run's cooled N_CS: Delta N_CS accumulated along the gradient flow as
    GradientFlow::CalibrationUpdate does (GradientFlow.cpp:168-188, improved E.B),
    every 10 steps of dtau 0.02, against the oracle (32^3, from the leapfrogged state)."""
    P = oracle_port[2]
    shape = (32, 32, 32)
    src = _cooling_input(ctx, shape, 200)
    U, E = src.download()
    lat = tcym.Lattice(ctx, 2, shape, prec)
    lat.copy_from(src)
    if prec == tcym.FP32:
        U, E = lat.download()
    got, ref = 0.0, 0.0
    scale = 0.0
    for _ in range(5):
        d = lat.flow(0.02, 10, tcym.FLOW_SIMULTANEOUS, calibrate=tcym.NCS_IMPROVED)
        r = P.flow(shape, U, E, 0.02, 10, 1)
        got, ref = got + d, ref + r
        scale = max(scale, abs(r))
        assert abs(got - ref) <= tol * max(scale, 1e-6), (got, ref)
