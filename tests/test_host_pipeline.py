"""The issue order of the host-resident step (tcym_leapfrog_host) on the CPU:
the library's own schedule, through the host check build, checked for every
chunk's whole stencil being on the device before the chunk is stepped.

Storage units are sites, or the site pairs (x, y, z) + (x, y, z + nz/2) of the
paired FP32 step; either way unit (x, y, z') has index x + nx (y + ny z') with
z' < nz' (nz, or nz/2 for pairs), and its stencil lies in the 3 x 3 x 3 block
around it, periodic in all three directions (for pairs, the wrap in z' is the
seam where neighbours arrive lane-swapped).
"""
import numpy as np
import pytest

from tests import _hostcheck as hc


def stencil_max(nx, ny, nzp, a, b):
    """Largest index in the 3x3x3 periodic neighbourhood of units [a, b)."""
    i = np.arange(a, b)
    x, y, z = i % nx, (i // nx) % ny, i // (nx * ny)
    m = -1
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                j = (x + dx) % nx + nx * ((y + dy) % ny + ny * ((z + dz) % nzp))
                m = max(m, int(j.max()))
    return m


def check_schedule(nx, ny, nzp, C):
    N, P = nx * ny * nzp, nx * ny
    b, ops = hc.pipeline_schedule(N, P, C)
    n = len(b) - 1
    assert b[0] == 0 and b[-1] == N and all(x < y for x, y in zip(b, b[1:]))
    assert all(x % 128 == 0 for x in b[:-1])  # the paired step's blocks start on chunk bounds
    assert all(y - x <= max(C, 128) for x, y in zip(b, b[1:]))
    assert sorted(j for k, j in ops if k == 0) == list(range(n))
    assert sorted(j for k, j in ops if k == 1) == list(range(n))
    up = 0  # uploads are in chunk order, so the units on the device are [0, up)
    expect_next = 0
    for kind, j in ops:
        lo, hi = b[j], b[j + 1]
        if kind == 0:
            assert j == expect_next
            expect_next += 1
            up = hi
            continue
        assert stencil_max(nx, ny, nzp, lo, hi) < up, (nx, ny, nzp, C, j, up)
    return b, ops


@pytest.mark.parametrize("nx,ny,nz", [(8, 8, 12), (8, 8, 9), (16, 16, 8), (12, 10, 14), (5, 6, 7), (128, 128, 128),
                                      (2, 2, 2), (96, 96, 96)])
@pytest.mark.parametrize("paired", [True, False])
@pytest.mark.parametrize("C", [128, 256, 1024, 13440, 53760, 1 << 20])
def test_schedule_respects_neighbourhoods(nx, ny, nz, paired, C):
    if paired and nz % 2:
        pytest.skip("the paired step needs an even nz")
    check_schedule(nx, ny, nz // 2 if paired else nz, C)


def test_schedule_overlaps_steps_with_uploads():
    """At 128^3 (paired, 64 MB chunks): one-plane chunks at both ends, so stepping
    starts after four planes are up and little is left to download after the
    last upload; steps start long before the last upload."""
    b, ops = check_schedule(128, 128, 64, 53760)
    P = 128 * 128
    first_step = next(i for i, (k, _) in enumerate(ops) if k == 1)
    uploads_before = sum(1 for k, _ in ops[:first_step] if k == 0)
    assert b[uploads_before] <= 4 * P
    last_upload = max(i for i, (k, _) in enumerate(ops) if k == 0)
    left = [j for k, j in ops[last_upload + 1:] if k == 1]
    assert sum(b[j + 1] - b[j] for j in left) <= 4 * P  # the last two planes' chunks and the first plane's
    assert last_upload > len(b)  # steps interleave with uploads


@pytest.mark.parametrize("nc,prec", [(2, "f32"), (3, "f32"), (3, "f64")])
@pytest.mark.parametrize("shape", [(8, 8, 12), (8, 8, 9), (16, 16, 8), (6, 10, 14)])
def test_pipeline_emulated_with_the_device_code(oracle_port, nc, prec, shape):
    """The library's schedule run with the device's own per-site code (the host check
    build): storage poisoned with NaN, each chunk converted in from the AoS arrays at its
    upload, each chunk stepped over its index range (the block offsets of the range
    launches) at its step; the stepped state equals the whole-lattice step bit for bit
    and holds no NaN, so no step read a neighbour before its upload."""
    import numpy as np

    import oracle

    P = oracle_port[nc]
    U, E = oracle.empty_fields(nc, shape)
    P.random_links(shape, U, 0.5, 3)
    P.gaussian_efield(shape, E, 0.7, 4)
    ref = hc.HostLattice(nc, prec, shape)
    ref.upload(U, E)
    ref.step(0, 0.05)  # the whole lattice, linear paired walk (or per site)
    want = ref.download()

    nx, ny, nz = shape
    V = nx * ny * nz
    paired = prec == "f32" and nz % 2 == 0
    N, Vh = ((V + 1) // 2 if paired else V), (V + 1) // 2
    H = hc.HostLattice(nc, prec, shape)
    H.poison()
    b, ops = hc.pipeline_schedule(N, nx * ny, 128)
    for kind, j in ops:
        lo, hi = b[j], b[j + 1]
        if kind == 0:
            H.from_aos_range(U, E, lo, hi - lo)
            if paired:
                H.from_aos_range(U, E, lo + Vh, hi - lo)
        else:
            H.step_range(0.05, lo, hi)
    H.cur ^= 1
    got = H.download()
    for g_, w_ in zip(got, want):
        assert not np.isnan(g_).any()
        assert np.array_equal(g_, w_)


def test_schedule_on_random_extents_and_chunks():
    """300 seeded random lattices (extents 1..20, paired or not) and chunk sizes."""
    import numpy as np

    rng = np.random.default_rng(11)
    for _ in range(300):
        nx, ny = int(rng.integers(1, 21)), int(rng.integers(1, 21))
        nzp = int(rng.integers(1, 13))
        C = 128 * int(rng.integers(1, 9))
        check_schedule(nx, ny, nzp, C)


def test_pipeline_emulated_on_random_shapes(oracle_port):
    """Eight seeded random shapes through the poisoned emulation (SU(2) FP32 and FP64)."""
    import numpy as np

    rng = np.random.default_rng(12)
    for k in range(8):
        shape = tuple(int(x) for x in rng.integers(3, 13, size=3))
        prec = "f32" if k % 2 == 0 else "f64"
        test_pipeline_emulated_with_the_device_code(oracle_port, 2, prec, shape)
