"""Host-side checks of the device arithmetic (no GPU needed).

* Philox4x32-10 against the published known-answer vectors (Salmon et al.,
  SC'11, Random123 distribution), in the oracle and in the device code.
* The per-site device functions, instantiated on the host by the test-only
  build (libtcym_hostcheck.so), against the FP64 oracle: FP64 formats to
  1e-12, FP32 formats to 1e-5 (the device-path tolerances).
"""
import numpy as np
import pytest

import oracle
from tests import _hostcheck as hc

KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]

FORMATS = [(2, "f64"), (2, "f32"), (3, "f64"), (3, "f32")]
TOL = {"f64": 1e-12, "f32": 1e-5}


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("ctr,key,out", KAT)
def test_philox_known_answers(oracle_port, ctr, key, out):
    assert tuple(oracle_port[2].philox(ctr, key)) == out


def test_device_normals_equal_oracle_normals(oracle_port):
    P = oracle_port[3]
    for seed, stream, step, site, mu, a in [(3, 0, 0, 0, 0, 0), (3, 0, 17, 4095, 2, 7), (1, 1, 0, 99, 1, 2),
                                            (2**40 + 5, 2, 2**33 + 1, 123456, 0, 5)]:
        ref = P.normal(seed, stream, step, site, mu, a)
        assert abs(hc.normal(seed, stream, step, site, mu, a) - ref) < 1e-15 * max(1, abs(ref))
        assert abs(hc.normal(seed, stream, step, site, mu, a, single=True) - ref) < 2e-6 * max(1, abs(ref))


def test_normal_stream_statistics(oracle_port):
    P = oracle_port[3]
    z = np.array([P.normal(9, 0, 0, s, mu, a) for s in range(400) for mu in range(3) for a in range(8)])
    assert abs(z.mean()) < 0.05 and abs(z.std() - 1.0) < 0.05


@pytest.mark.parametrize("nc,prec", FORMATS)
def test_exponential(oracle_port, nc, prec):
    P = oracle_port[nc]
    rng = np.random.default_rng(5)
    for scale in (1e-6, 1e-3, 0.1, 1.0, 3.0, 10.0):
        for _ in range(10):
            al = rng.normal(size=oracle.NA[nc]) * scale
            c = float(rng.normal())
            assert np.abs(hc.iexp(nc, prec, c, al) - P.matrix_iexp(c, al)).max() < 10 * TOL[prec]


def _state(P, nc, shape, seed):
    U, E = oracle.empty_fields(nc, shape)
    P.random_links(shape, U, 0.6, seed)
    P.gaussian_efield(shape, E, 0.7, seed + 1)
    return U, E


@pytest.mark.parametrize("nc,prec", FORMATS)
def test_site_step_leapfrog_langevin_flow(oracle_port, nc, prec):
    P = oracle_port[nc]
    shape = (4, 5, 6)
    U, E = _state(P, nc, shape, 3)
    H = hc.HostLattice(nc, prec, shape)
    H.upload(U, E)
    H.leapfrog(0.05, 10)
    P.leapfrog(shape, U, E, 0.05, 10)
    Uh, Eh = H.download()
    assert rel(Uh, U) < TOL[prec] and rel(Eh, E) < TOL[prec]
    H.langevin(0.02, 1.0, 0.6, 3, 0, 5)
    P.langevin(shape, U, E, 0.02, 1.0, 0.6, 3, 0, 5)
    Uh, Eh = H.download()
    assert rel(Uh, U) < TOL[prec] and rel(Eh, E) < TOL[prec]
    H.flow(0.02, 3)
    P.flow(shape, U, E, 0.02, 3, 0)
    Uh, Eh = H.download()
    assert rel(Uh, U) < TOL[prec] and rel(Eh, E) < TOL[prec]


@pytest.mark.parametrize("nc", [2, 3])
@pytest.mark.parametrize("shape", [(8, 8, 16), (6, 4, 2), (5, 5, 5)])
def test_site_pair_step(oracle_port, nc, shape):
    """The FP32 formats' paired step against the oracle and against the per-site
    step on the same paired layout: (8,8,16) has seam and interior blocks of
    128 pairs; at nz = 2 a pair's partner is its own z-neighbour; odd V (5^3)
    has a padding site and no paired step."""
    P = oracle_port[nc]
    U, E = _state(P, nc, shape, 21)
    H = hc.HostLattice(nc, "f32", shape)
    S = hc.HostLattice(nc, "f32", shape)
    S.pairs = 0
    for X in (H, S):
        X.upload(U, E)
        X.leapfrog(0.05, 5)
        X.langevin(0.02, 1.0, 0.6, 7, 0, 3)
    P.leapfrog(shape, U, E, 0.05, 5)
    P.langevin(shape, U, E, 0.02, 1.0, 0.6, 7, 0, 3)
    Uh, Eh = H.download()
    Us, Es = S.download()
    assert rel(Uh, U) < 1e-5 and rel(Eh, E) < 1e-5
    assert rel(Uh, Us) < 1e-5 and rel(Eh, Es) < 1e-5


@pytest.mark.parametrize("nc,prec", FORMATS)
def test_site_checkerboard_flow(oracle_port, nc, prec):
    P = oracle_port[nc]
    shape = (4, 4, 6)
    U, E = _state(P, nc, shape, 9)
    H = hc.HostLattice(nc, prec, shape)
    H.upload(U, E)
    H.flow_checkerboard(0.05, 2)
    P.flow_checkerboard(shape, U, 0.05, 2)
    assert rel(H.download()[0], U) < TOL[prec]


@pytest.mark.parametrize("nc,prec", FORMATS)
def test_site_observables_and_restore(oracle_port, nc, prec):
    P = oracle_port[nc]
    shape = (4, 5, 6)
    U, E = _state(P, nc, shape, 13)
    H = hc.HostLattice(nc, prec, shape)
    H.upload(U, E)
    Ur, Er = H.download()
    o, r = H.observables(), P.observables(shape, Ur, Er)
    for k in list(range(14)) + [15]:
        assert abs(o[k] - r[k]) < TOL[prec] * max(1.0, abs(r[k])), oracle.OBS_FIELDS[k]
    if prec == "f64":
        it_h = H.gauss_restore(1e-14, 10000)
        it_o = P.gauss_restore(shape, U, E, 1e-14, 10000)
        assert abs(it_h - it_o) <= 1
        assert rel(H.download()[1], E) < 1e-12


@pytest.mark.parametrize("shape", [(4, 5, 6), (6, 4, 8), (5, 6, 2)])
@pytest.mark.parametrize("nc", [2, 3])
def test_paired_edotb_sample(oracle_port, nc, shape):
    """The N_CS sample of FP32 pair storage through the paired code (both sites of a
    pair in packed FP32, the z seam's lane swaps) against the per-site code and the
    oracle on the same (FP32-rounded) state: E^2 and B^2 within 1e-7, clover E.B (a sum
    that cancels) within 1e-7 of V |E| |B|, the scale of the sum of |E.B| over the
    sites (measured: 1e-9 and 5e-10 at most)."""
    P = oracle_port[nc]
    U, E = _state(P, nc, shape, 19)
    H = hc.HostLattice(nc, "f32", shape)
    H.upload(U, E)
    Ur, Er = H.download()
    got, per_site, ref = H.edotb_pair(), H.observables(mask=8), P.observables(shape, Ur, Er)
    assert got is not None
    scale = np.prod(shape) * 2.0 * np.sqrt(ref[1] * ref[2])  # V |E| |B|
    for k in (1, 2, 3, 4, 5, 6, 7, 8):
        assert abs(got[k] - ref[k]) < 1e-7 * max(1.0, abs(ref[k])), (k, got[k], ref[k])
        assert abs(got[k] - per_site[k]) < 1e-7 * max(1.0, abs(per_site[k])), (k, got[k], per_site[k])
    assert abs(got[13] - ref[13]) < 1e-7 * max(scale, abs(ref[13])), (got[13], ref[13], scale)
    assert abs(got[13] - per_site[13]) < 1e-7 * max(scale, abs(per_site[13]))


def test_fp32_flow_keeps_link_norms_unbiased(oracle_port):
    """100 checkerboard sweeps (dtau 0.02) of an SU(2) 8^3 lattice in FP32 storage, the
    device's site code on the host, against the FP64 oracle from the same rounded start:
    the magnetic energy (it falls from 1.2 to 2e-3 a site) within 2e-4.  With the link
    update as exp * u, cos(d/2) rounding next to 1 moved every norm the same way and
    the error was 7.9e-4 here (0.18 after 500 sweeps at 96^3); in increment form 3.6e-5."""
    P = oracle_port[2]
    shape = (8, 8, 8)
    U, E = oracle.empty_fields(2, shape)
    P.random_links(shape, U, 0.7, 5)
    H = hc.HostLattice(2, "f32", shape)
    H.upload(U, E)
    U, E = H.download()
    H.flow_checkerboard(0.02, 100)
    P.flow_checkerboard(shape, U, 0.02, 100)
    o, r = H.observables(), P.observables(shape, U, E)
    assert abs(o[2] - r[2]) < 2e-4 * r[2], (o[2], r[2])


@pytest.mark.parametrize("nc,prec", FORMATS)
def test_site_improved_edotb(oracle_port, nc, prec):
    P = oracle_port[nc]
    shape = (4, 5, 6)
    U, E = _state(P, nc, shape, 17)
    H = hc.HostLattice(nc, prec, shape)
    H.upload(U, E)
    Ur, Er = H.download()
    ref = P.edotb_improved(shape, Ur, Er)
    assert abs(H.observables(mask=16)[13] - ref) < TOL[prec] * max(1.0, abs(ref))


@pytest.mark.parametrize("nc", [2, 3])
def test_reunitarize_restores_group(oracle_port, nc):
    P = oracle_port[nc]
    shape = (3, 3, 4)
    U, E = _state(P, nc, shape, 21)
    U = U * (1 + 1e-3 * np.random.default_rng(1).normal(size=U.shape))  # drift off the group
    H = hc.HostLattice(nc, "f64", shape)
    H.upload(U, E)
    assert H.observables()[11] > 1e-4
    H.reunitarize()
    assert H.observables()[11] < 1e-14


@pytest.mark.parametrize("nc", [2, 3])
@pytest.mark.parametrize("shape", [(3, 3, 4), (3, 3, 3)])  # even volume; odd volume (a padded pair)
def test_fp32_reunitarize_matches_fp64(oracle_port, nc, shape):
    """FP32 links are widened to FP64, projected and rounded back: the FP64
    lattice's result to a few FP32 ulps (the input was rounded to FP32 first,
    and row 2 of SU(3) is rebuilt in FP32), on the group to FP32 rounding."""
    P = oracle_port[nc]
    U, E = _state(P, nc, shape, 22)
    U = U * (1 + 1e-3 * np.random.default_rng(2).normal(size=U.shape))
    H32, H64 = hc.HostLattice(nc, "f32", shape), hc.HostLattice(nc, "f64", shape)
    H32.upload(U, E)
    H64.upload(U, E)
    assert H32.observables()[11] > 1e-4
    H32.reunitarize()
    H64.reunitarize()
    assert H32.observables()[11] < 1e-6
    U32, _ = H32.download()
    U64, _ = H64.download()
    assert np.abs(U32 - U64).max() < 3e-7


@pytest.mark.parametrize("nc", [2, 3])
def test_initial_conditions(oracle_port, nc):
    P = oracle_port[nc]
    shape = (3, 4, 5)
    U, E = oracle.empty_fields(nc, shape)
    P.random_links(shape, U, 0.3, 2)
    P.gaussian_efield(shape, E, 0.5, 1)
    H = hc.HostLattice(nc, "f64", shape)
    H.init(2, 0.3, 2)
    H.init(1, 0.5, 1)
    Uh, Eh = H.download()
    assert rel(Eh, E) < 1e-15 and rel(Uh, U) < 1e-13


@pytest.mark.parametrize("nc", [2, 3])
def test_matrix_log(oracle_port, nc):
    """The device matrix log (host build, FP64) against the oracle's, and exp(log V) = V:
    generic elements, small rotations (the geodesic's case), the identity, elements
    with degenerate eigenvalues, and rotations near the branch cut (eigenphases ~ pi)."""
    P = oracle_port[nc]
    rng = np.random.default_rng(8)
    na = 3 if nc == 2 else 8
    cases = [rng.normal(size=na) * s for s in (1e-6, 0.05, 0.5, 1.5) for _ in range(4)]
    cases.append(np.zeros(na))
    if nc == 3:
        cases += [np.array([0, 0, 1.2, 0, 0, 0, 0, 0.0]), np.array([0, 0, 0, 0, 0, 0, 0, 2.0]),
                  np.array([0, 0, 0.9, 0, 0, 0, 0, 0.9 / np.sqrt(3)])]  # two equal eigenphases
    else:
        cases += [np.array([0, 0, 2 * np.pi - 1e-3])]
    for a in cases:
        v = P.matrix_iexp(-1.0, a)
        got, ref = hc.ilog(nc, "f64", -1.0, v), P.ilog(-1.0, v)
        assert np.abs(got - ref).max() < 1e-9 * max(1.0, np.abs(ref).max()), (a, got, ref)
        assert np.abs(P.matrix_iexp(-1.0, got) - v).max() < 1e-12


@pytest.mark.parametrize("nc,prec", FORMATS)
def test_site_geodesic(oracle_port, nc, prec):
    """GeodesicInterpolation on every link: UMid and EMid against the oracle."""
    P = oracle_port[nc]
    shape = (4, 4, 6)
    Uo, _ = oracle.empty_fields(nc, shape)
    Un, _ = oracle.empty_fields(nc, shape)
    P.random_links(shape, Uo, 0.4, 12)
    P.random_links(shape, Un, 0.4, 13)
    A, B, M = (hc.HostLattice(nc, prec, shape) for _ in range(3))
    A.upload(Uo, None)
    B.upload(Un, None)
    if prec == "f32":  # the oracle starts from the rounded links
        Uo, Un = A.download()[0], B.download()[0]
    for c in (0.0, 0.5, 1.0):
        M.geodesic(A, B, c)
        Um, Em = P.geodesic(shape, Uo, Un, c)
        Uh, Eh = M.download()
        assert rel(Uh, Um) < TOL[prec] and rel(Eh, Em) < TOL[prec]
    assert rel(M.download()[0], Un) < TOL[prec]  # c = 1 lands on UNew


@pytest.mark.parametrize("nc", [2, 3])
def test_pair_step_tilings(oracle_port, nc):
    """Every block tiling of the paired step (linear, and tx x 128/tx tiles of one z-plane,
    including tiles wider than the lattice) visits each pair once with the right seam
    handling: the results are bit-identical across tilings and match the oracle."""
    P = oracle_port[nc]
    shape = (12, 10, 8)
    U, E = _state(P, nc, shape, 41)
    out = []
    for tx in (0, 128, 32, 16, 8):
        H = hc.HostLattice(nc, "f32", shape)
        H.pairs = 1 + tx
        H.upload(U, E)
        H.leapfrog(0.05, 3)
        out.append(H.download())
    for Uh, Eh in out[1:]:
        assert np.array_equal(Uh, out[0][0]) and np.array_equal(Eh, out[0][1])
    P.leapfrog(shape, U, E, 0.05, 3)
    assert rel(out[0][0], U) < 1e-5 and rel(out[0][1], E) < 1e-5


@pytest.mark.parametrize("nc,prec", FORMATS)
def test_block_matches_oracle(oracle_port, nc, prec):
    """The device's Block (site_block: U_mu(2x) U_mu(2x + mu) in FP64) on the host, on
    the stored links, against the oracle's."""
    P = oracle_port[nc]
    shape = (4, 6, 8)
    U, E = _state(P, nc, shape, 23)
    H = hc.HostLattice(nc, prec, shape)
    H.upload(U, E)
    Us, _ = H.download()  # the stored (for FP32: rounded) links
    B = hc.HostLattice(nc, prec, (2, 3, 4))
    H.block_into(B)
    Ub, _ = B.download()
    assert np.abs(Ub - P.block(shape, Us)).max() < (1e-14 if prec == "f64" else 3e-7)


@pytest.mark.parametrize("nc,prec", FORMATS)
def test_parity_bounds_catch_a_planted_error(oracle_port, nc, prec):
    """The parity bounds are tight enough to see a mistake: the same comparison as
    test_site_step_leapfrog_langevin_flow, with an error planted in the oracle's run
    (its time step off by 1e-4, and a Langevin noise seed off by one), fails them."""
    P = oracle_port[nc]
    shape = (4, 5, 6)
    U, E = _state(P, nc, shape, 3)
    H = hc.HostLattice(nc, prec, shape)
    H.upload(U, E)
    H.leapfrog(0.05, 10)
    Ub, Eb = U.copy(), E.copy()
    P.leapfrog(shape, Ub, Eb, 0.05 * (1 + 1e-4), 10)
    Uh, Eh = H.download()
    assert max(rel(Uh, Ub), rel(Eh, Eb)) > TOL[prec]
    P.leapfrog(shape, U, E, 0.05, 10)
    H.langevin(0.02, 1.0, 0.6, 3, 0, 2)
    P.langevin(shape, U, E, 0.02, 1.0, 0.6, 4, 0, 2)
    Uh, Eh = H.download()
    assert max(rel(Uh, U), rel(Eh, E)) > TOL[prec]
