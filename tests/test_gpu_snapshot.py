"""Binary snapshots: stop a run, restore it into a fresh lattice, and the continuation
is bit-identical to the run that never stopped.

The runs cross the periodic FP64 reunitarisation (every 100 steps), track the
Kahan-compensated N_CS every step, and (for Langevin) continue the Philox noise
stream from the step the snapshot recorded, so every counter of the resume is
exercised.  The reference can only checkpoint through its 15-digit configuration
text files (IO/SaveConfiguration.cpp:3-56), which do not resume FP32 storage exactly.
"""
import numpy as np
import pytest

import oracle
import topologicalcymsolver_gb300 as tcym

pytestmark = pytest.mark.gpu

PREC = [pytest.param(tcym.FP32, id="fp32"), pytest.param(tcym.FP64, id="fp64")]
GROUPS = [pytest.param(2, id="su2"), pytest.param(3, id="su3")]


def _start(nc, shape, seed):
    P = oracle.Port(nc)
    U, E = oracle.empty_fields(nc, shape)
    P.random_links(shape, U, 0.3, seed)
    P.gaussian_efield(shape, E, 0.7, seed + 1)
    return U, E


def _run(lat, mode, n, step0):
    if mode == "leapfrog":
        lat.leapfrog(0.05, n)
    else:
        lat.langevin(0.02, 1.0, 0.6, 3, step0, n)


@pytest.mark.parametrize("mode", ["leapfrog", "langevin"])
@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
def test_snapshot_resume_is_bit_identical(ctx, nc, prec, mode, tmp_path):
    oracle.build()
    shape = (8, 6, 10)
    U, E = _start(nc, shape, 31)
    N, M = 70, 60  # the reunitarisation at step 100 falls after the snapshot

    def fresh():
        lat = tcym.Lattice(ctx, nc, shape, prec)
        lat.set_reunitarize_period(100)
        lat.ncs_track(1)
        return lat

    # the uninterrupted run
    a = fresh()
    a.upload(U, E)
    _run(a, mode, N + M, 0)
    Ua, Ea = a.download()
    ncs_a = a.ncs()
    a.close()

    # N steps, snapshot (in memory and to a file), restore into fresh lattices, M steps
    b = fresh()
    b.upload(U, E)
    _run(b, mode, N, 0)
    snap = b.snapshot()
    path = tmp_path / "lattice.snap"
    b.snapshot_file(path)
    assert path.read_bytes() == bytes(snap)
    b.close()
    for restore in ("buffer", "file"):
        c = tcym.Lattice(ctx, nc, shape, prec)  # untracked, default period: the snapshot sets both
        c.set_reunitarize_period(7)
        if restore == "buffer":
            c.restore(snap)
        else:
            c.restore_file(path)
        assert c.steps() == N
        seed, nxt, ok = c.noise_state()
        step0 = 0
        if mode == "langevin":
            assert ok and seed == 3 and nxt == N
            step0 = nxt
        _run(c, mode, M, step0)
        Uc, Ec = c.download()
        assert np.array_equal(Uc, Ua) and np.array_equal(Ec, Ea), restore
        assert c.ncs() == ncs_a  # the Kahan pair resumed exactly
        assert c.steps() == N + M
        c.close()


def test_snapshot_rejects_other_lattices_and_corruption(ctx):
    oracle.build()
    U, E = _start(3, (6, 6, 6), 41)
    a = tcym.Lattice(ctx, 3, (6, 6, 6), tcym.FP32)
    a.upload(U, E)
    snap = a.snapshot()
    for nc, shape, prec in ((3, (6, 6, 8), tcym.FP32), (3, (6, 6, 6), tcym.FP64), (2, (6, 6, 6), tcym.FP32)):
        other = tcym.Lattice(ctx, nc, shape, prec)
        with pytest.raises(tcym.TcymError) as ei:
            other.restore(snap)
        assert ei.value.code == 1
        other.close()
    bad = bytearray(snap)
    bad[len(bad) // 2] ^= 0x40
    with pytest.raises(tcym.TcymError) as ei:
        a.restore(bad)
    assert ei.value.code == 1 and "checksum" in str(ei.value)
    with pytest.raises(tcym.TcymError):
        a.restore(snap[: len(snap) - 16])
    a.restore(snap)  # the intact snapshot still restores
    Ua, Ea = a.download()
    a.close()
