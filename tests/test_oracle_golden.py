"""The oracle (FP64 C restatement) pinned against the reference's own outputs.

Fixtures under tests/golden/ were produced by the reference's sources compiled
in place (tests/golden/make_golden.py).  The oracle must reproduce them to
FP64 rounding: 1e-12 relative for single steps and observables; 1e-10 after
100 leapfrog steps (the SU(3) exponential uses another eigensolver, so
rounding differs at 1e-16 per step and grows slowly in the chaotic dynamics).
"""
import os

import numpy as np
import pytest

import oracle

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def load(name):
    return dict(np.load(os.path.join(G, name)))


@pytest.mark.parametrize("nc", [2, 3])
def test_group_kats(oracle_port, nc):
    P = oracle_port[nc]
    d = load(f"ref_group_su{nc}.npz")
    for i in range(len(d["c"])):
        assert np.abs(P.matrix_iexp(d["c"][i], d["alpha"][i]) - d["exp"][i]).max() < 2e-14
        assert np.abs(P.retr_igen(d["exp"][i] * 1.1) - d["proj"][i]).max() < 1e-15
        assert np.abs(P.adjoint(d["exp"][i], d["e"][i]) - d["adj"][i]).max() < 1e-14
        assert np.abs(P.inverse_adjoint(d["exp"][i], d["e"][i]) - d["iadj"][i]).max() < 1e-14


@pytest.mark.parametrize("nc", [2, 3])
def test_states_leapfrog(oracle_port, nc):
    P = oracle_port[nc]
    d = load(f"ref_states_su{nc}.npz")
    shape = tuple(d["shape"])
    U, E = d["U0"].copy(), d["E0"].copy()
    for n, tag, tol in ((1, "lf1", 1e-13), (9, "lf10", 1e-12), (90, "lf100", 1e-10)):
        P.leapfrog(shape, U, E, 0.05, n)
        assert rel(U, d["U_" + tag]) < tol
        assert rel(E, d["E_" + tag]) < tol
        o = P.observables(shape, U, E)
        r = d["obs_" + tag]
        for k in range(15):
            assert abs(o[k] - r[k]) < 1e-9 * max(1.0, abs(r[k])), (tag, oracle.OBS_FIELDS[k])


@pytest.mark.parametrize("nc", [2, 3])
def test_states_langevin_same_noise(oracle_port, nc):
    P = oracle_port[nc]
    d = load(f"ref_states_su{nc}.npz")
    shape = tuple(d["shape"])
    U, E = d["U0"].copy(), d["E0"].copy()
    P.langevin(shape, U, E, 0.02, 1.0, 0.6, 3, 0, 10)
    assert rel(U, d["U_lv10"]) < 1e-12
    assert rel(E, d["E_lv10"]) < 1e-12


@pytest.mark.parametrize("nc", [2, 3])
def test_states_flow_and_calibration(oracle_port, nc):
    P = oracle_port[nc]
    d = load(f"ref_states_su{nc}.npz")
    shape = tuple(d["shape"])
    U, E = d["U0"].copy(), d["E0"].copy()
    P.flow(shape, U, E, 0.02, 10, 0)
    assert rel(U, d["U_fl10"]) < 1e-12
    assert rel(E, d["E_fl10"]) < 1e-12
    o = P.observables(shape, U, E)
    for k in (13, 14):  # clover and O(a^2)-improved E.B of the flowed state
        assert abs(o[k] - d["obs_fl10"][k]) < 1e-10 * max(1.0, abs(d["obs_fl10"][k]))
    # CalibrationUpdate's Delta N_CS with the reference's NCsDot (improved operator)
    U, E = d["U0"].copy(), d["E0"].copy()
    dn = P.flow(shape, U, E, 0.02, 10, 1)
    assert abs(dn - float(d["dncs_fl10"])) < 1e-12 * max(1.0, abs(float(d["dncs_fl10"])))


@pytest.mark.parametrize("nc", [2, 3])
def test_states_gauss_restore(oracle_port, nc):
    P = oracle_port[nc]
    d = load(f"ref_states_su{nc}.npz")
    shape = tuple(d["shape"])
    U, E = d["U0"].copy(), d["E0"].copy()
    P.gauss_restore(shape, U, E)
    assert rel(E, d["E_gr"]) < 1e-12
    o = P.observables(shape, U, E)
    assert o[9] <= 1e-14 * 10 and d["obs_gr"][9] <= 1e-13


@pytest.mark.parametrize("nc", [2, 3])
def test_observables_of_inputs(oracle_port, nc):
    P = oracle_port[nc]
    d = load(f"ref_states_su{nc}.npz")
    shape = tuple(d["shape"])
    o = P.observables(shape, d["U0"], d["E0"])
    r = d["obs_0"]
    for k in range(15):
        assert abs(o[k] - r[k]) < 1e-12 * max(1.0, abs(r[k])), oracle.OBS_FIELDS[k]


def test_su2_16_leapfrog_initial_state_and_series(oracle_port):
    """The SU(2) 16^3 leapfrog run: the oracle's IC equals the reference's, and the
    first 100 steps of the energy series agree pointwise."""
    P = oracle_port[2]
    d = load("ref_leapfrog_su2_16.npz")
    shape = (16, 16, 16)
    U, E = oracle.empty_fields(2, shape)
    P.set_zero(shape, U, E)
    P.gaussian_efield(shape, E, 1.0 / np.sqrt(2.0), 1)
    P.gauss_restore(shape, U, E, 1e-14, 10000)
    assert rel(E, d["E_ic"]) < 1e-12
    s = d["series"]
    o = P.observables(shape, U, E)
    assert abs(o[0] - s[0][0]) < 1e-12
    for rec in range(1, 11):  # 10 records = 100 steps
        P.leapfrog(shape, U, E, 0.05, 10)
        o = P.observables(shape, U, E)
        assert abs(o[0] - s[rec][0]) < 1e-10 * s[rec][0]
        assert abs(o[13] - s[rec][13]) < 1e-8 * max(1.0, abs(s[rec][13]))


@pytest.mark.parametrize("nc", [2, 3])
def test_thermalize_equals_reference(oracle_port, nc):
    """ThermalDynamics::Thermalize: the oracle's restatement reproduces the
    reference's final fields and its ThermalEnergy series (written with 6 digits)."""
    d = load(f"ref_thermalize_su{nc}.npz")
    shape = tuple(int(v) for v in d["shape"])
    P = oracle_port[nc]
    U, E = oracle.empty_fields(nc, shape)
    P.set_zero(shape, U, E)
    series = P.thermalize(shape, U, E, float(d["beta"]), int(d["seed"]), int(d["rounds"]), float(d["max_time"]),
                          float(d["dtau"]), 20)
    assert series.shape == d["series"].shape
    assert np.allclose(series, d["series"], rtol=5e-6, atol=1e-6)
    assert rel(U, d["U"]) < 1e-12 and rel(E, d["E"]) < 1e-12


def test_cooled_delta_ncs_equals_reference(oracle_port):
    """ChernSimonsNumber::CoolingMethod (SU(2), where the reference's matrix log needs
    no LAPACK): the oracle's cooling, geodesic and Simpson rule reproduce the
    reference's cumulative cooled Delta N_CS and its cooled links."""
    d = load("ref_cooling_su2.npz")
    P = oracle_port[2]
    shape = (6, 6, 6)
    U, E = d["U0"].copy(), d["E0"].copy()
    steps, s = int(d["steps"]), float(d["sqrt_dctau"])
    old = U.copy()
    P.cool(shape, old, s, steps)
    total = 0.0
    for k in range(3):
        P.leapfrog(shape, U, E, float(d["dt"]), int(d["every"]))
        new = U.copy()
        P.cool(shape, new, s, steps)
        total += P.cooled_delta_ncs(shape, old, new, 1)
        assert abs(total - d["totals"][k]) < 1e-12, (k, total, d["totals"][k])
        assert rel(new, d["cooled"][k]) < 1e-12
        old = new


@pytest.mark.parametrize("level", [1, 2])
def test_blocked_cooling_equals_reference(oracle_port, level):
    """CoolingMethod with StandardBlockingLevel 1 and 2 (Cooling::Perform's Blocks after
    steps BlockFrequency 8^b, each doubling the spacing): the oracle's blocked cooling
    reproduces the reference's cooled links on the blocked extents and its ΔN_CS."""
    d = load("ref_cooling_blocked_su2.npz")
    P = oracle_port[2]
    shape = (8, 8, 8)
    small = tuple(k >> level for k in shape)
    U, E = d["U0"].copy(), d["E0"].copy()
    steps, bf, s = int(d[f"steps{level}"]), int(d[f"bf{level}"]), float(d["sqrt_dctau"])
    old = P.cool_blocked(shape, U, s, steps, level, bf)
    total = 0.0
    for k in range(3):
        P.leapfrog(shape, U, E, float(d["dt"]), int(d["every"]))
        new = P.cool_blocked(shape, U, s, steps, level, bf)
        total += P.cooled_delta_ncs(small, old, new, 1)
        assert rel(new, d[f"cooled{level}"][k]) < 1e-12
        assert abs(total - d[f"totals{level}"][k]) < 1e-12, (k, total, d[f"totals{level}"][k])
        old = new


@pytest.mark.parametrize("nc", [2, 3])
def test_blocked_cooling_composes_flow_and_block(oracle_port, nc):
    """The oracle's blocked cooling equals its own pieces: bf flow steps, Block, the
    remaining steps at the same dtau (the spacing factors cancel), for both groups."""
    P = oracle_port[nc]
    shape = (4, 4, 6)
    U, E = oracle.empty_fields(nc, shape)
    P.random_links(shape, U, 0.5, 9)
    s, steps, bf = 0.15, 7, 3
    got = P.cool_blocked(shape, U, s, steps, 1, bf)
    W, F = U.copy(), np.zeros_like(E)
    P.flow(shape, W, F, s * s, bf, 0)
    Wb = P.block(shape, W)
    small = (2, 2, 3)
    _, Fb = oracle.empty_fields(nc, small)
    P.flow(small, Wb, Fb, s * s, steps - bf, 0)
    assert np.abs(got - Wb).max() < 1e-13


def test_block_is_the_product_of_two_links(oracle_port):
    """Block(GaugeLinks**) on SU(3): U'_mu(x) = U_mu(2x) U_mu(2x + mu), checked link by link."""
    P = oracle_port[3]
    shape = (4, 6, 2)
    U, _ = oracle.empty_fields(3, shape)
    P.random_links(shape, U, 0.6, 7)
    Ub = P.block(shape, U)
    nx, ny = shape[0], shape[1]

    def mat(v):
        return (v[0::2] + 1j * v[1::2]).reshape(3, 3, order="F")  # column-major complex 3x3

    for (x, y, z) in [(0, 0, 0), (1, 2, 0), (1, 1, 0)]:
        s0 = 2 * x + nx * (2 * y + ny * 2 * z)
        sb = x + (nx // 2) * (y + (ny // 2) * z)
        for mu, step in enumerate((1, nx, nx * ny)):
            s1 = s0 + step if mu < 2 or 2 * z + 1 < shape[2] else s0 + step - nx * ny * shape[2]
            ref = mat(U[s0, mu]) @ mat(U[s1, mu])
            assert np.abs(mat(Ub[sb, mu]) - ref).max() < 1e-14


@pytest.mark.parametrize("level", [0, 1])
def test_su3_cooling_equals_reference(oracle_port, level):
    """SU(3) CoolingMethod (level 0 at 6^3, blocking level 1 at 8^3), the reference's own
    with its MatrixILog calling LAPACK's ZGEEV (OpenBLAS 0.3.31 as SciPy ships it): the
    oracle's cooled links and cumulative cooled Delta N_CS equal it."""
    d = load("ref_cooling_su3.npz")
    P = oracle_port[3]
    U, E = d[f"U0_{level}"].copy(), d[f"E0_{level}"].copy()
    shape = {0: (6, 6, 6), 1: (8, 8, 8)}[level]
    small = tuple(k >> level for k in shape)
    steps, bf, s = int(d[f"steps{level}"]), int(d[f"bf{level}"]), float(d["sqrt_dctau"])
    old = P.cool_blocked(shape, U, s, steps, level, bf)
    total = 0.0
    for k in range(3):
        P.leapfrog(shape, U, E, float(d["dt"]), int(d["every"]))
        new = P.cool_blocked(shape, U, s, steps, level, bf)
        total += P.cooled_delta_ncs(small, old, new, 1)
        assert rel(new, d[f"cooled{level}"][k]) < 1e-12
        assert abs(total - d[f"totals{level}"][k]) < 1e-11, (k, total, d[f"totals{level}"][k])
        old = new


@pytest.mark.parametrize("zgeev", ["restated", "lapack"])
def test_su3_matrix_log_equals_reference(oracle_port, monkeypatch, zgeev):
    """The reference's SU(3) MatrixILog, its ZGEEV either restated or LAPACK's (SciPy's
    OpenBLAS), against the oracle's log on elements up to and across the branch cut at
    angle pi."""
    if not oracle.ref_available(3):
        pytest.skip("the reference's sources are compiled only where they are present")
    R = oracle.Ref(3)
    P = oracle_port[3]
    if zgeev == "lapack":
        lapack = oracle.scipy_lapack()
        if lapack is None:
            pytest.skip("no LAPACK with ZGEEV found")
        monkeypatch.setenv("TCYM_REF_LAPACK", lapack[0])
    else:
        monkeypatch.delenv("TCYM_REF_LAPACK", raising=False)
    assert R.lapack_in_use() == (zgeev == "lapack")
    rng = np.random.default_rng(3)
    for scale in (1e-3, 0.1, 1.0, 3.0):
        for _ in range(10):
            V = P.matrix_iexp(1.0, rng.normal(size=8) * scale)
            assert np.abs(R.matrix_ilog(1.0, V) - P.ilog(1.0, V)).max() < 1e-12
    # degenerate eigenvalues: the identity, and exp(i theta t_8) (two equal phases)
    for al in (np.zeros(8), np.eye(8)[7] * 1.3, np.eye(8)[7] * -2.2 + np.eye(8)[2] * 1e-9):
        V = P.matrix_iexp(1.0, al)
        assert np.abs(R.matrix_ilog(1.0, V) - P.ilog(1.0, V)).max() < 1e-9
