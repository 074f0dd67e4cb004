"""Ensembles (tcym_ensemble_*): members of mixed group, size, precision and
dynamics advanced in batched, graph-captured launches.

* each member ends where the same lattice stepped alone ends, bit for bit;
* a member's state, E.B and N_CS are bit-identical alone in an ensemble and in a mix;
* chunks of different lengths and membership changes rebuild the graph correctly;
* the persistent K-step launches give the same bits as one launch per step, with one
  member group or many;
* members against the FP64 oracle directly (FP64 <= 1e-10, FP32 <= 1e-5 over 100 steps).
"""
import numpy as np
import pytest

import oracle
import topologicalcymsolver_gb300 as tcym

pytestmark = pytest.mark.gpu

SPECS = [  # (nc, shape, precision, dynamics)
    (2, (4, 5, 6), tcym.FP64, tcym.DYN_LEAPFROG),
    (3, (6, 6, 6), tcym.FP64, tcym.DYN_LANGEVIN),
    (3, (5, 4, 7), tcym.FP32, tcym.DYN_LEAPFROG),
    (2, (8, 8, 8), tcym.FP32, tcym.DYN_LANGEVIN),
    (3, (4, 4, 4), tcym.FP32, tcym.DYN_LANGEVIN),
    (2, (6, 5, 4), tcym.FP64, tcym.DYN_LANGEVIN),
]


def make(ctx, P, nc, shape, prec, seed):
    U, E = oracle.empty_fields(nc, shape)
    P.random_links(shape, U, 0.6, seed)
    P.gaussian_efield(shape, E, 0.7, seed + 1)
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.set_reunitarize_period(0)
    lat.upload(U, E)
    return lat


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_members_match_lattices_stepped_alone(ctx, oracle_port):
    ens = tcym.Ensemble(ctx)
    pairs = []
    for i, (nc, shape, prec, dyn) in enumerate(SPECS):
        a = make(ctx, oracle_port[nc], nc, shape, prec, 100 + i)
        b = make(ctx, oracle_port[nc], nc, shape, prec, 100 + i)
        ens.add(a, 0.05 if dyn == tcym.DYN_LEAPFROG else 0.02, dyn, 1.0, 0.6, 7 + i, 0)
        pairs.append((a, b, dyn, i))
    ens.step(5)
    ens.step(5)
    ens.step(3)  # a chunk of another length: the graph is rebuilt
    for a, b, dyn, i in pairs:
        if dyn == tcym.DYN_LEAPFROG:
            b.leapfrog(0.05, 13)
        else:
            b.langevin(0.02, 1.0, 0.6, 7 + i, 0, 13)
        Ua, Ea = a.download()
        Ub, Eb = b.download()
        # the same per-site (per-pair) arithmetic with the same coefficients: the same bits
        assert np.array_equal(Ua, Ub) and np.array_equal(Ea, Eb), (i, rel(Ua, Ub), rel(Ea, Eb))
    edb, _ = ens.measure()
    for (a, _, _, _), e in zip(pairs, edb):
        assert abs(e - a.edotb()) < 1e-9 * max(1.0, abs(e))


def test_member_bit_identical_alone_and_in_mix(ctx, oracle_port):
    nc, shape, prec = 3, (6, 5, 6), tcym.FP32
    P = oracle_port[nc]
    solo = tcym.Ensemble(ctx)
    x = make(ctx, P, nc, shape, prec, 55)
    solo.add(x, 0.02, tcym.DYN_LANGEVIN, 1.0, 0.6, 3, 0)
    mix = tcym.Ensemble(ctx)
    y = make(ctx, P, nc, shape, prec, 55)
    others = [make(ctx, oracle_port[s[0]], s[0], s[1], s[2], 300 + j) for j, s in enumerate(SPECS)]
    for j, o in enumerate(others[:3]):
        mix.add(o, 0.05, tcym.DYN_LEAPFROG)
    mix.add(y, 0.02, tcym.DYN_LANGEVIN, 1.0, 0.6, 3, 0)
    for o in others[3:]:
        mix.add(o, 0.02, tcym.DYN_LANGEVIN, 1.0, 0.5, 9, 0)
    n1, n2 = [], []
    for _ in range(4):
        solo.step(20)
        mix.step(20)
        n1.append(solo.measure(20))
        n2.append(mix.measure(20))
    Ux, Ex = x.download()
    Uy, Ey = y.download()
    assert np.array_equal(Ux, Uy) and np.array_equal(Ex, Ey)
    k = 3  # y's position in the mix
    for (e1, c1), (e2, c2) in zip(n1, n2):
        assert e1[0] == e2[k] and c1[0] == c2[k]


def test_membership_changes(ctx, oracle_port):
    ens = tcym.Ensemble(ctx)
    lats = [make(ctx, oracle_port[2], 2, (4, 4, 4), tcym.FP64, 900 + i) for i in range(3)]
    ref = [make(ctx, oracle_port[2], 2, (4, 4, 4), tcym.FP64, 900 + i) for i in range(3)]
    for L in lats:
        ens.add(L, 0.05)
    ens.step(4)
    ens.remove(lats[1])
    assert len(ens) == 2
    ens.step(4)
    ref[0].leapfrog(0.05, 8)
    ref[1].leapfrog(0.05, 4)
    ref[2].leapfrog(0.05, 8)
    for L, R in zip(lats, ref):
        assert np.array_equal(L.download()[0], R.download()[0])
    with pytest.raises(tcym.TcymError):
        ens.add(lats[0], 0.05)  # already a member


PERSISTENT_SPECS = [  # (nc, shape, precision, dynamics): paired FP32 members take the persistent launch
    (3, (8, 8, 8), tcym.FP32, tcym.DYN_LEAPFROG),
    (2, (16, 16, 16), tcym.FP32, tcym.DYN_LEAPFROG),
    (3, (12, 10, 8), tcym.FP32, tcym.DYN_LANGEVIN),
    (2, (6, 6, 4), tcym.FP32, tcym.DYN_LANGEVIN),
    (3, (16, 16, 16), tcym.FP32, tcym.DYN_LEAPFROG),
    (3, (6, 6, 6), tcym.FP32, tcym.DYN_LEAPFROG),
    (3, (5, 4, 7), tcym.FP32, tcym.DYN_LEAPFROG),  # odd nz: per-site, one launch per step
    (2, (6, 5, 4), tcym.FP64, tcym.DYN_LANGEVIN),  # FP64: one launch per step
]


@pytest.mark.parametrize("group_blocks", [0, 4])
def test_persistent_launches_match_per_step_launches(ctx, oracle_port, group_blocks):
    runs = {}
    for mode in ("launches", "persistent"):
        ens = tcym.Ensemble(ctx)
        if mode == "persistent":
            ens.set_persistent(group_blocks)
        lats = []
        for i, (nc, shape, prec, dyn) in enumerate(PERSISTENT_SPECS):
            lat = make(ctx, oracle_port[nc], nc, shape, prec, 400 + i)
            ens.add(lat, 0.05 if dyn == tcym.DYN_LEAPFROG else 0.02, dyn, 1.0, 0.6, 11 + i, 0)
            lats.append(lat)
        ncs = []
        for chunk in (20, 20, 7):
            ens.step(chunk)
            ncs.append(ens.measure(chunk))
        runs[mode] = ([lat.download() for lat in lats], ncs)
        ens.close()
        for lat in lats:
            lat.close()
    (sa, na), (sb, nb) = runs["launches"], runs["persistent"]
    for i, ((Ua, Ea), (Ub, Eb)) in enumerate(zip(sa, sb)):
        assert np.array_equal(Ua, Ub) and np.array_equal(Ea, Eb), i
    for (ea, ca), (eb, cb) in zip(na, nb):
        assert np.array_equal(ea, eb) and np.array_equal(ca, cb)


def test_members_against_oracle(ctx, oracle_port):
    """Members stepped in a (persistent) ensemble against the oracle fed the same start
    and noise: FP64 <= 1e-10, FP32 <= 1e-5 relative over 100 steps."""
    specs = [(2, (8, 6, 10), tcym.FP32, tcym.DYN_LEAPFROG), (3, (6, 6, 8), tcym.FP32, tcym.DYN_LANGEVIN),
             (3, (6, 6, 6), tcym.FP64, tcym.DYN_LEAPFROG), (2, (6, 8, 6), tcym.FP64, tcym.DYN_LANGEVIN),
             (3, (8, 8, 8), tcym.FP32, tcym.DYN_LEAPFROG)]
    ens = tcym.Ensemble(ctx)
    ens.set_persistent(0)
    members = []
    for i, (nc, shape, prec, dyn) in enumerate(specs):
        P = oracle_port[nc]
        U, E = oracle.empty_fields(nc, shape)
        P.random_links(shape, U, 0.3, 600 + i)
        P.gaussian_efield(shape, E, 0.7, 700 + i)
        lat = tcym.Lattice(ctx, nc, shape, prec)
        lat.set_reunitarize_period(0)
        lat.upload(U, E)
        if prec == tcym.FP32:  # the oracle starts from the stored (rounded) state
            U, E = lat.download()
        dt = 0.05 if dyn == tcym.DYN_LEAPFROG else 0.02
        ens.add(lat, dt, dyn, 1.0, 0.6, 800 + i, 0)
        members.append((lat, P, nc, shape, prec, dyn, dt, U, E, 800 + i))
    for _ in range(5):
        ens.step(20)
    for lat, P, nc, shape, prec, dyn, dt, U, E, seed in members:
        if dyn == tcym.DYN_LEAPFROG:
            P.leapfrog(shape, U, E, dt, 100)
        else:
            P.langevin(shape, U, E, dt, 1.0, 0.6, seed, 0, 100)
        Ug, Eg = lat.download()
        tol = 1e-10 if prec == tcym.FP64 else 1e-5
        print(f"measured ensemble member SU({nc}) {shape} prec={prec} dyn={dyn}: U {rel(Ug, U):.2e} E {rel(Eg, E):.2e}")
        assert rel(Ug, U) < tol and rel(Eg, E) < tol, (nc, shape, prec, dyn, rel(Ug, U), rel(Eg, E))
    ens.close()
