"""Lattice blocking on the GPU: tcym_lattice_block (Block(GaugeLinks**),
Block(ElectricFields**)) against the oracle, and cooling with
StandardBlockingLevel 1 and 2 (tcym_cooling_create_ex) against the
reference's own CoolingMethod outputs (tests/golden/ref_cooling_blocked_su2.npz)
and the oracle for SU(3)."""
import os

import numpy as np
import pytest

import oracle
import topologicalcymsolver_gb300 as tcym

pytestmark = pytest.mark.gpu

PREC = [pytest.param(tcym.FP64, id="fp64"), pytest.param(tcym.FP32, id="fp32")]
GROUPS = [pytest.param(2, id="su2"), pytest.param(3, id="su3")]
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_cooling_blocked_su2.npz")


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
def test_block_matches_oracle(ctx, oracle_port, nc, prec):
    P = oracle_port[nc]
    shape = (4, 6, 8)
    U, E = oracle.empty_fields(nc, shape)
    P.random_links(shape, U, 0.6, 7)
    P.gaussian_efield(shape, E, 0.7, 8)
    src = tcym.Lattice(ctx, nc, shape, prec)
    src.upload(U, E)
    U, _ = src.download()  # the stored (for FP32: rounded) links
    dst = tcym.Lattice(ctx, nc, (2, 3, 4), prec)
    dst.gaussian_efield(0.7, 9)  # overwritten by zeros
    src.block_into(dst)
    Ub, Eb = dst.download()
    assert rel(Ub, P.block(shape, U)) < (1e-14 if prec == tcym.FP64 else 2e-7)
    assert not Eb.any()
    # the source is unchanged and can be blocked again
    U2, _ = src.download()
    assert np.array_equal(U2, U)


def test_block_rejects_bad_shapes(ctx):
    src = tcym.Lattice(ctx, 2, (4, 4, 4), tcym.FP32)
    for shape, prec in (((2, 2, 3), tcym.FP32), ((2, 2, 2), tcym.FP64)):
        with pytest.raises(tcym.TcymError) as ei:
            src.block_into(tcym.Lattice(ctx, 2, shape, prec))
        assert ei.value.code == 1
    odd = tcym.Lattice(ctx, 2, (4, 4, 5), tcym.FP32)
    with pytest.raises(tcym.TcymError):
        odd.block_into(tcym.Lattice(ctx, 2, (2, 2, 2), tcym.FP32))


def test_blocked_cooling_rejects_unreachable_levels(ctx):
    lat = tcym.Lattice(ctx, 2, (8, 8, 12), tcym.FP32)
    for level, steps, bf in ((1, 16, 0), (2, 7, 1), (3, 128, 1), (1, 1, 2)):  # no frequency, 8 > 7, 12 % 8, 2 > 1
        with pytest.raises(tcym.TcymError) as ei:
            tcym.Cooling(lat, steps, 0.1, level, bf)
        assert ei.value.code == 1


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("level", [1, 2])
def test_blocked_cooling_matches_reference(ctx, prec, level):
    """SU(2) 8^3, Start then three rounds of 20 leapfrog steps and Update(1): the
    cumulative cooled Delta N_CS and the cooled links on the blocked extents, against
    the reference's CoolingMethod with StandardBlockingLevel = level."""
    d = np.load(GOLDEN)
    lat = tcym.Lattice(ctx, 2, (8, 8, 8), prec)
    lat.set_reunitarize_period(0)
    lat.upload(d["U0"], d["E0"])
    steps, bf = int(d[f"steps{level}"]), int(d[f"bf{level}"])
    cool = tcym.Cooling(lat, steps, float(d["sqrt_dctau"]), level, bf)
    cool.start()
    totals = d[f"totals{level}"]
    scale = float(np.abs(np.diff(np.concatenate([[0.0], totals]))).max())
    for k in range(3):
        lat.leapfrog(float(d["dt"]), int(d["every"]))
        cool.update(True)
        links = cool.links()
        assert links.shape[0] == 512 >> (3 * level)
        if prec == tcym.FP64:
            assert rel(links, d[f"cooled{level}"][k]) < 1e-10
            assert abs(cool.total() - totals[k]) < 1e-10 * max(scale, 1e-3)
        else:
            assert rel(links, d[f"cooled{level}"][k]) < 1e-4
            assert abs(cool.total() - totals[k]) < 1e-3 * max(scale, 1e-3), (k, cool.total(), totals[k])
    cool.close()


@pytest.mark.parametrize("prec", PREC)
def test_blocked_cooling_su3_matches_oracle(ctx, oracle_port, prec):
    """SU(3) 8^3 at StandardBlockingLevel 1: the device's cooled links and Delta N_CS
    against the oracle's blocked cooling (the oracle equals the reference's own, run on
    LAPACK's ZGEEV, in the golden tests)."""
    P = oracle_port[3]
    shape = (8, 8, 8)
    U, E = oracle.empty_fields(3, shape)
    P.random_links(shape, U, 0.4, 11)
    P.gaussian_efield(shape, E, 0.6, 12)
    P.gauss_restore(shape, U, E, 1e-14, 10000)
    lat = tcym.Lattice(ctx, 3, shape, prec)
    lat.set_reunitarize_period(0)
    lat.upload(U, E)
    if prec == tcym.FP32:
        U, E = lat.download()
    s, steps, bf = np.sqrt(0.02), 12, 2
    cool = tcym.Cooling(lat, steps, s, 1, bf)
    cool.start()
    old = P.cool_blocked(shape, U, s, steps, 1, bf)
    for _ in range(2):
        lat.leapfrog(0.05, 10)
        P.leapfrog(shape, U, E, 0.05, 10)
        new = P.cool_blocked(shape, U, s, steps, 1, bf)
        ref = P.cooled_delta_ncs((4, 4, 4), old, new, 1)
        got = cool.update(True)
        tol = 1e-9 if prec == tcym.FP64 else 1e-3
        assert abs(got - ref) <= tol * max(abs(ref), 1e-3), (got, ref)
        assert rel(cool.links(), new) < (1e-10 if prec == tcym.FP64 else 1e-4)
        old = new
    cool.close()
