"""GPU parity: the sm_103a kernels through the C ABI against the FP64 oracle.

Tolerances (the accuracy contract): FP64 device path <= 1e-10 relative over short
windows (<= 100 steps), FP32 storage path <= 1e-5 relative.  "Relative" is the
max-abs difference over the max-abs magnitude of the oracle's array.
"""
import numpy as np
import pytest

import oracle
import topologicalcymsolver_gb300 as tcym

pytestmark = pytest.mark.gpu

TOL = {tcym.FP64: 1e-10, tcym.FP32: 1e-5}
PREC = [pytest.param(tcym.FP64, id="fp64"), pytest.param(tcym.FP32, id="fp32")]
GROUPS = [pytest.param(2, id="su2"), pytest.param(3, id="su3")]


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def random_state(P, nc, shape, seed=3, sigma_u=0.6, sigma_e=0.7):
    U, E = oracle.empty_fields(nc, shape)
    P.random_links(shape, U, sigma_u, seed)
    P.gaussian_efield(shape, E, sigma_e, seed + 1)
    return U, E


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
@pytest.mark.parametrize("shape", [(6, 6, 6), (5, 6, 7)])
@pytest.mark.parametrize("sigma_u", [0.6, 0.3], ids=["rough", "thermal"])
def test_leapfrog_parity(ctx, oracle_port, nc, prec, shape, sigma_u):
    """FP64 <= 1e-10, FP32 <= 1e-5 relative.  The rough start (link angles of width
    0.6) is chaotic enough to amplify FP32 storage rounding ~6x per 50 steps (measured
    5e-7 at step 10, 9e-6 at step 100), so it is compared through step 10; the start
    with the configurations' width 0.3 through step 100."""
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, sigma_u=sigma_u)
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.set_reunitarize_period(0)
    lat.upload(U, E)
    checks = ((1, 1), (10, 9)) if sigma_u > 0.5 else ((1, 1), (10, 9), (100, 90))  # cumulative steps, dt 0.05
    for total, nsteps in checks:
        lat.leapfrog(0.05, nsteps)
        P.leapfrog(shape, U, E, 0.05, nsteps)
        Ug, Eg = lat.download()
        tol = TOL[prec]
        print(f"measured leapfrog SU({nc}) {shape} prec={prec} sigma_u={sigma_u} step {total}: "
              f"U {rel(Ug, U):.2e} E {rel(Eg, E):.2e}")
        assert rel(Ug, U) < tol, (total, rel(Ug, U))
        assert rel(Eg, E) < tol, (total, rel(Eg, E))


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
def test_split_updates_parity(ctx, oracle_port, nc, prec):
    """Dynamics::UpdateElectricFields and UpdateGaugeLinks called separately."""
    shape = (4, 6, 5)
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=11)
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.upload(U, E)
    lat.update_e(0.03)
    P.update_e(shape, U, E, 0.03)
    Ug, Eg = lat.download()
    assert rel(Eg, E) < TOL[prec]
    lat.update_u(0.03)
    P.update_u(shape, U, E, 0.03)
    Ug, Eg = lat.download()
    assert rel(Ug, U) < TOL[prec]


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
def test_langevin_parity_same_noise(ctx, oracle_port, nc, prec):
    shape = (6, 5, 6)
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=21)
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.set_reunitarize_period(0)
    lat.upload(U, E)
    lat.langevin(0.02, 1.0, 0.6, 3, 0, 20)
    P.langevin(shape, U, E, 0.02, 1.0, 0.6, 3, 0, 20)
    Ug, Eg = lat.download()
    assert rel(Ug, U) < TOL[prec]
    assert rel(Eg, E) < TOL[prec]


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
def test_flow_parity(ctx, oracle_port, nc, prec):
    shape = (6, 6, 4)
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=31)
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.upload(U, E)
    d_gpu = lat.flow(0.02, 5, tcym.FLOW_SIMULTANEOUS, calibrate=tcym.NCS_IMPROVED)
    d_orc = P.flow(shape, U, E, 0.02, 5, 1)
    Ug, Eg = lat.download()
    assert rel(Ug, U) < TOL[prec]
    assert rel(Eg, E) < TOL[prec]
    assert abs(d_gpu - d_orc) < TOL[prec] * max(abs(d_orc), 1e-3) * 10
    # checkerboard sweeps (in place, parity x direction order)
    lat.flow(0.02, 3, tcym.FLOW_CHECKERBOARD)
    P.flow_checkerboard(shape, U, 0.02, 3)
    Ug, _ = lat.download()
    assert rel(Ug, U) < TOL[prec]


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
def test_observables_parity(ctx, oracle_port, nc, prec):
    shape = (5, 6, 4)
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=41)
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.upload(U, E)
    if prec == tcym.FP32:  # compare against the oracle on the rounded state
        U, E = lat.download()
    o = lat.observables().as_oracle_vector()
    r = P.observables(shape, U, E)
    tol = 1e-12 if prec == tcym.FP64 else 1e-5
    for k in list(range(0, 11)) + [13, 15]:
        assert abs(o[k] - r[k]) <= tol * max(1.0, abs(r[k])), (oracle.OBS_FIELDS[k], o[k], r[k])
    # unitarity: FP32 links carry rounding at 1e-7
    assert abs(o[11] - r[11]) <= (1e-12 if prec == tcym.FP64 else 1e-6)


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
def test_improved_edotb_parity(ctx, oracle_port, nc, prec):
    shape = (5, 4, 6)
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=43)
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.upload(U, E)
    U, E = lat.download()
    ref = P.edotb_improved(shape, U, E)
    tol = 1e-12 if prec == tcym.FP64 else 1e-5
    assert abs(lat.edotb_improved() - ref) < tol * max(1.0, abs(ref))
    assert abs(lat.edotb() - P.edotb_clover(shape, U, E)) < tol * max(1.0, abs(ref))


@pytest.mark.parametrize("nc", GROUPS)
def test_initial_conditions_match_oracle(ctx, oracle_port, nc):
    shape = (4, 5, 6)
    P = oracle_port[nc]
    U, E = oracle.empty_fields(nc, shape)
    P.random_links(shape, U, 0.3, 2)
    P.gaussian_efield(shape, E, np.sqrt(0.5), 1)
    lat = tcym.Lattice(ctx, nc, shape, tcym.FP64)
    lat.random_links(0.3, 2)
    lat.gaussian_efield(np.sqrt(0.5), 1)
    Ug, Eg = lat.download()
    assert rel(Eg, E) < 1e-14
    assert rel(Ug, U) < 1e-13
    lat.set_zero()
    P.set_zero(shape, U, E)
    Ug, Eg = lat.download()
    assert np.array_equal(Ug, U) and np.array_equal(Eg, E)


@pytest.mark.parametrize("nc", GROUPS)
def test_gauss_restore(ctx, oracle_port, nc):
    shape = (6, 6, 6)
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=51)
    lat = tcym.Lattice(ctx, nc, shape, tcym.FP64)
    lat.upload(U, E)
    it_g, mx = lat.gauss_restore(1e-14, 10000)
    it_o = P.gauss_restore(shape, U, E, 1e-14, 10000)
    Ug, Eg = lat.download()
    assert abs(it_g - it_o) <= 1  # the max crosses tol at the same iteration up to rounding
    assert rel(Eg, E) < 1e-10
    o = P.observables(shape, Ug, Eg)
    assert o[9] <= 1e-13 and o[15] < 1e-12


@pytest.mark.parametrize("shape", [(6, 6, 6), (5, 6, 7)], ids=["paired", "odd_nz"])
@pytest.mark.parametrize("nc", GROUPS)
def test_gauss_restore_fp32_against_oracle(ctx, oracle_port, nc, shape):
    """FP32 storage: 8 restore iterations (tol 0, so both run them all; the absolute
    maximum falls from ~5 to ~5e-4) against the FP64 oracle's from the same state.  Even
    nz takes the paired FP32 kernels (packed pairs, FP32 arithmetic and scratch), odd nz
    the per-site kernels (FP64 accumulation): the fields within 1e-5 of their scale, the
    restored state's violation (signed max and absolute max) within 1e-5 of the oracle's."""
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=57)
    lat = tcym.Lattice(ctx, nc, shape, tcym.FP32)
    lat.upload(U, E)
    it_g, _ = lat.gauss_restore(0.0, 8)
    it_o = P.gauss_restore(shape, U, E, 0.0, 8)
    Ug, Eg = lat.download()
    err = rel(Eg, E)
    o = P.observables(shape, U, E)
    og = lat.observables()
    dg = max(abs(og.gauss_max - o[9]), abs(og.gauss_absmax - o[15]))
    print(f"\nmeasured FP32 restore SU({nc}) {shape}: E {err:.2e}, violation {dg:.2e} of {o[15]:.3e}")
    assert it_g == 8 and it_o == 8
    assert err < 1e-5
    assert dg < 1e-5 * max(1.0, abs(o[15]))
    lat.close()


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
def test_gauss_restore_reports_nan(ctx, oracle_port, nc, prec):
    """A NaN in E: the signed maximum drops it (fmax), the sums keep it; the restore
    must fail with TCYM_ERR_NONFINITE, and a clean restore afterwards must succeed."""
    shape = (6, 6, 6)
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=53)
    bad = E.copy()
    bad[5, 2, 1] = np.nan
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.upload(U, bad)
    with pytest.raises(tcym.TcymError) as ei:
        lat.gauss_restore(1e-14, 10000)
    assert ei.value.code == 4
    lat.upload(U, E)
    lat.gauss_restore(1e-6 if prec == tcym.FP32 else 1e-14, 10000)
    lat.close()


@pytest.mark.parametrize("nc", GROUPS)
def test_upload_download_roundtrip(ctx, oracle_port, nc):
    shape = (3, 4, 5)
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape)
    lat = tcym.Lattice(ctx, nc, shape, tcym.FP64)
    lat.upload(U, E)
    Ug, Eg = lat.download()
    assert np.array_equal(Ug, U) and np.array_equal(Eg, E)
    lat32 = tcym.Lattice(ctx, nc, shape, tcym.FP32)
    lat32.upload(U, E)
    Ug, Eg = lat32.download()
    assert rel(Ug, U) < 2e-7 and rel(Eg, E) < 1e-7


@pytest.mark.parametrize("nc", GROUPS)
@pytest.mark.parametrize("shape", [(4, 6, 6), (3, 5, 7)])  # even volume; odd volume (a padded last pair)
def test_reunitarize_fp32_vs_fp64(ctx, oracle_port, nc, shape):
    """Links drifted off the group: the FP64 lattice's Gram-Schmidt puts them on
    the group to 1e-14; the FP32 lattice's (FP64 arithmetic on the FP32 links)
    agrees with it to a few FP32 ulps and is on the group to FP32 rounding."""
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape)
    U = U * (1 + 1e-3 * np.random.default_rng(4).normal(size=U.shape))
    lat64 = tcym.Lattice(ctx, nc, shape, tcym.FP64)
    lat32 = tcym.Lattice(ctx, nc, shape, tcym.FP32)
    lat64.upload(U, E)
    lat32.upload(U, E)
    assert lat32.observables().unit_max > 1e-4
    lat64.reunitarize()
    lat32.reunitarize()
    assert lat64.observables().unit_max < 1e-14
    assert lat32.observables().unit_max < 1e-6
    U64, _ = lat64.download()
    U32, _ = lat32.download()
    assert np.abs(U32 - U64).max() < 3e-7


@pytest.mark.parametrize("nc", GROUPS)
def test_ncs_tracking_is_kahan_sum_of_edotb(ctx, oracle_port, nc):
    shape = (6, 6, 6)
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=61)
    lat = tcym.Lattice(ctx, nc, shape, tcym.FP64)
    lat.upload(U, E)
    lat.ncs_track(1)
    lat.ncs_reset()
    dt, total = 0.05, 0.0
    for _ in range(10):
        lat.leapfrog(dt, 1)
        P.leapfrog(shape, U, E, dt, 1)
        total += dt * P.edotb_clover(shape, U, E) / (8 * np.pi ** 2)
    assert abs(lat.ncs() - total) < 1e-11 * max(1.0, abs(total))


@pytest.mark.parametrize("shape", [(6, 6, 6), (4, 6, 5)], ids=["paired", "odd_nz"])
@pytest.mark.parametrize("nc", GROUPS)
def test_ncs_tracking_fp32_against_oracle(ctx, oracle_port, nc, shape):
    """FP32 storage, N_CS sampled every 2 steps (the paired E.B kernel for even nz, the
    per-site one for odd nz) against the oracle's Kahan-free sum of dt * 2 * clover
    E.B / 8 pi^2 over the same 20 steps from the same (FP32-rounded) state: within
    2e-8 of the sum's scale, 20 dt V |E| |B| / 8 pi^2 (measured 1.3e-10 .. 1.1e-9)."""
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=63, sigma_u=0.3)
    lat = tcym.Lattice(ctx, nc, shape, tcym.FP32)
    lat.set_reunitarize_period(0)
    lat.upload(U, E)
    U, E = lat.download()
    lat.ncs_track(2)
    lat.ncs_reset()
    dt, total = 0.05, 0.0
    for _ in range(10):
        lat.leapfrog(dt, 2)
        P.leapfrog(shape, U, E, dt, 2)
        total += 2 * dt * P.edotb_clover(shape, U, E) / (8 * np.pi ** 2)
    o = P.observables(shape, U, E)
    scale = 20 * dt * np.prod(shape) * 2.0 * np.sqrt(o[1] * o[2]) / (8 * np.pi ** 2)
    err = abs(lat.ncs() - total) / scale
    print(f"\nmeasured FP32 N_CS tracking SU({nc}) {shape}: {err:.2e} of {scale:.3e}")
    assert err < 2e-8


def test_error_codes(ctx):
    with pytest.raises(tcym.TcymError) as ei:
        tcym.Lattice(ctx, 4, (4, 4, 4))
    assert ei.value.code == 1
    lat = tcym.Lattice(ctx, 2, (5, 4, 4))
    with pytest.raises(tcym.TcymError) as ei:
        lat.flow(0.01, 1, tcym.FLOW_CHECKERBOARD)  # odd extent
    assert ei.value.code == 1


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
def test_thermalize_parity(ctx, oracle_port, nc, prec):
    """tcym_thermalize against the oracle's ThermalDynamics::Thermalize (2 rounds of
    20 steps at dTau 0.0375 from U = 1, records every 5 steps)."""
    shape = (6, 4, 6)
    P = oracle_port[nc]
    U, E = oracle.empty_fields(nc, shape)
    P.set_zero(shape, U, E)
    ref = P.thermalize(shape, U, E, 2.0, 7, 2, 0.75, 0.0375, 5)
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.set_zero()
    series = lat.thermalize(2.0, 7, 2, 0.75, 0.0375, every=5)
    assert series.shape == ref.shape == (8, 7)
    tol = TOL[prec]  # measured FP32: series 2e-7, fields 9e-7
    Ug, Eg = lat.download()
    print(f"\nmeasured thermalize SU({nc}) prec={prec}: series {np.abs(series - ref).max() / np.abs(ref).max():.2e} "
          f"U {rel(Ug, U):.2e} E {rel(Eg, E):.2e}")
    assert np.abs(series - ref).max() <= tol * np.abs(ref).max()
    assert rel(Ug, U) < tol and rel(Eg, E) < tol


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
def test_cooled_delta_ncs_parity(ctx, oracle_port, nc, prec):
    """tcym_cooling_* against the oracle's CoolingMethod: Start, then three rounds of
    20 leapfrog steps and Update(1) with 16 cooling steps; the cumulative cooled
    Delta N_CS after each update and GetDeltaNCs(2) on the last pair."""
    shape = (6, 6, 6)
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=3, sigma_u=0.5)
    P.gauss_restore(shape, U, E, 1e-14, 10000)
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.set_reunitarize_period(0)
    lat.upload(U, E)
    if prec == tcym.FP32:
        U, E = lat.download()
    s, steps = np.sqrt(0.02), 16
    cool = tcym.Cooling(lat, steps, s)
    cool.start()
    old = U.copy()
    P.cool(shape, old, s, steps)
    total, scale = 0.0, 0.0
    for _ in range(3):
        lat.leapfrog(0.05, 20)
        P.leapfrog(shape, U, E, 0.05, 20)
        new = U.copy()
        P.cool(shape, new, s, steps)
        d = P.cooled_delta_ncs(shape, old, new, 1)
        total += d
        scale = max(scale, abs(d))
        got = cool.update(True)
        # a sum that cancels: relative to the largest increment (measured FP32: 1.0e-6 of it)
        tol = 1e-9 if prec == tcym.FP64 else 1e-5
        print(f"measured cooled Delta N_CS SU({nc}) prec={prec}: |got-d| {abs(got - d):.2e} "
              f"scale {max(scale, 1e-3):.2e} total {abs(cool.total() - total):.2e}")
        assert abs(got - d) <= tol * max(scale, 1e-3), (got, d)
        assert abs(cool.total() - total) <= 3 * tol * max(scale, 1e-3)
        old = new
    ref2 = P.cooled_delta_ncs(shape, old, new, 2)
    assert abs(cool.delta_ncs(2) - ref2) <= (1e-9 if prec == tcym.FP64 else 1e-5) * max(abs(ref2), 1e-3)
    cool.close()


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
def test_configuration_files_round_trip(ctx, oracle_port, tmp_path, nc, prec):
    """tcym_lattice_save writes what tcym_write_configuration writes for the downloaded
    state; tcym_lattice_load of those files restores it (FP64: to the 15 digits of the
    format; FP32: the stored values exactly)."""
    shape = (4, 3, 6)
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=31)
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.upload(U, E)
    Ud, Ed = lat.download()
    lat.save(tmp_path / "U.txt", tmp_path / "E.txt")
    tcym.write_configuration(nc, shape, Ud, Ed, tmp_path / "U2.txt", tmp_path / "E2.txt")
    assert (tmp_path / "U.txt").read_bytes() == (tmp_path / "U2.txt").read_bytes()
    assert (tmp_path / "E.txt").read_bytes() == (tmp_path / "E2.txt").read_bytes()
    other = tcym.Lattice(ctx, nc, shape, prec)
    other.set_zero()
    other.load(tmp_path / "U.txt", tmp_path / "E.txt")
    U2, E2 = other.download()
    tol = 1e-14 if prec == tcym.FP64 else 0.0
    assert np.abs(U2 - Ud).max() <= tol and np.abs(E2 - Ed).max() <= tol * np.abs(Ed).max()


@pytest.mark.parametrize("nc", GROUPS)
def test_step_tilings_identical(ctx, oracle_port, nc):
    """The packed FP32 step's block tilings (linear and tx x ty tiles, one wider than the
    lattice) give bit-identical results; the autotuner picks one of the candidates."""
    shape = (24, 20, 16)
    P = oracle_port[nc]
    U, E = random_state(P, nc, shape, seed=51)
    results = []
    for tx in (0, 32, 16, 8, 128):
        lat = tcym.Lattice(ctx, nc, shape, tcym.FP32)
        lat.set_tile(tx, 0 if tx == 0 else 128 // tx)
        lat.upload(U, E)
        lat.leapfrog(0.05, 4)
        lat.langevin(0.02, 1.0, 0.6, 3, 0, 2)
        results.append(lat.download())
        lat.close()
    for Ug, Eg in results[1:]:
        assert np.array_equal(Ug, results[0][0]) and np.array_equal(Eg, results[0][1])
    auto = tcym.Lattice(ctx, nc, shape, tcym.FP32)
    tx, ty = auto.tile()
    assert tx == 0 or (tx * ty == 128 and tx <= shape[0] and ty <= shape[1])
    with pytest.raises(tcym.TcymError):
        auto.set_tile(48, 2)
