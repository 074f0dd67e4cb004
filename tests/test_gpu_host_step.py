"""tcym_leapfrog_host (one step of a host-resident state, transfers pipelined
with the step) against upload + tcym_leapfrog(1) + download: identical bit for
bit, for every format, paired and per-site steps, one and many chunks, in place
and out of place, and with a reunitarisation falling due."""
import numpy as np
import pytest

import oracle
import topologicalcymsolver_gb300 as tcym

pytestmark = pytest.mark.gpu

PREC = [pytest.param(tcym.FP64, id="fp64"), pytest.param(tcym.FP32, id="fp32")]
GROUPS = [pytest.param(2, id="su2"), pytest.param(3, id="su3")]


def state(P, nc, shape, seed):
    U, E = oracle.empty_fields(nc, shape)
    P.random_links(shape, U, 0.4, seed)
    P.gaussian_efield(shape, E, 0.7, seed + 1)
    return U, E


def sequential(ctx, nc, shape, prec, U, E, dt, nsteps, reunit=0):
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.set_reunitarize_period(reunit)
    for _ in range(nsteps):
        lat.upload(U, E)
        lat.leapfrog(dt, 1)
        U, E = lat.download()
    return U, E


@pytest.mark.parametrize("prec", PREC)
@pytest.mark.parametrize("nc", GROUPS)
# even nz: the paired FP32 step; odd nz: the per-site step; P = 256 > 128-unit chunks; odd volume
@pytest.mark.parametrize("shape", [(8, 8, 12), (8, 8, 9), (16, 16, 8), (5, 6, 7)])
@pytest.mark.parametrize("chunk", [128, 0])  # 0: the library's ~64 MB chunks (one chunk here)
def test_host_step_equals_upload_step_download(ctx, oracle_port, monkeypatch, nc, prec, shape, chunk):
    if chunk:
        monkeypatch.setenv("TCYM_HOST_STEP_CHUNK", str(chunk))
    else:
        monkeypatch.delenv("TCYM_HOST_STEP_CHUNK", raising=False)
    U, E = state(oracle_port[nc], nc, shape, 7)
    Us, Es = sequential(ctx, nc, shape, prec, U.copy(), E.copy(), 0.05, 3)
    lat = tcym.Lattice(ctx, nc, shape, prec)
    lat.set_reunitarize_period(0)
    Uh, Eh = U.copy(), E.copy()
    for _ in range(3):
        Uh, Eh = lat.leapfrog_host(0.05, Uh, Eh)
    assert np.array_equal(Uh, Us) and np.array_equal(Eh, Es)
    Ud, Ed = lat.download()  # the lattice holds the new state too
    assert np.array_equal(Ud, Us) and np.array_equal(Ed, Es)


@pytest.mark.parametrize("nc", GROUPS)
def test_host_step_in_place_many_chunks(ctx, oracle_port, monkeypatch, nc):
    """U_out = U_in, E_out = E_in, 12 chunks of 128 pairs (32 x 16 x 6)."""
    monkeypatch.setenv("TCYM_HOST_STEP_CHUNK", "128")
    shape = (32, 16, 6)
    U, E = state(oracle_port[nc], nc, shape, 9)
    Us, Es = sequential(ctx, nc, shape, tcym.FP32, U.copy(), E.copy(), 0.04, 2)
    lat = tcym.Lattice(ctx, nc, shape, tcym.FP32)
    lat.set_reunitarize_period(0)
    for _ in range(2):
        out = lat.leapfrog_host(0.04, U, E, U, E)
        assert out[0] is U and out[1] is E
    assert np.array_equal(U, Us) and np.array_equal(E, Es)


def test_host_step_default_chunks_at_96(ctx, oracle_port, monkeypatch):
    """SU(3) FP32 96^3 with the library's chunk size (9 chunks of 53760 pairs)."""
    monkeypatch.delenv("TCYM_HOST_STEP_CHUNK", raising=False)
    shape = (96, 96, 96)
    U, E = state(oracle_port[3], 3, shape, 11)
    Us, Es = sequential(ctx, 3, shape, tcym.FP32, U.copy(), E.copy(), 0.05, 1)
    lat = tcym.Lattice(ctx, 3, shape, tcym.FP32)
    lat.set_reunitarize_period(0)
    Uh, Eh = lat.leapfrog_host(0.05, U, E)
    assert np.array_equal(Uh, Us) and np.array_equal(Eh, Es)


@pytest.mark.parametrize("nc", GROUPS)
def test_host_step_with_reunitarisation_due(ctx, oracle_port, nc):
    shape = (8, 8, 8)
    U, E = state(oracle_port[nc], nc, shape, 13)
    Us, Es = sequential(ctx, nc, shape, tcym.FP32, U.copy(), E.copy(), 0.05, 4, reunit=2)
    lat = tcym.Lattice(ctx, nc, shape, tcym.FP32)
    lat.set_reunitarize_period(2)
    Uh, Eh = U.copy(), E.copy()
    for _ in range(4):
        Uh, Eh = lat.leapfrog_host(0.05, Uh, Eh)
    assert np.array_equal(Uh, Us) and np.array_equal(Eh, Es)


def test_host_step_rejects_bad_arrays(ctx):
    lat = tcym.Lattice(ctx, 2, (4, 4, 4), tcym.FP32)
    U, E = oracle.empty_fields(2, (4, 4, 4))
    with pytest.raises(ValueError):
        lat.leapfrog_host(0.05, U[:10], E)
    with pytest.raises(ValueError):
        lat.leapfrog_host(0.05, U.astype(np.float32), E)


@pytest.mark.parametrize("nc", GROUPS)
def test_host_step_pinned_graph_replay(ctx, oracle_port, monkeypatch, nc):
    """Pinned host arrays take the captured-graph pipeline: replays over both
    ping-pong parities, a new dt and new arrays (recaptures) all match the
    three-call sequence."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("TCYM_HOST_STEP_CHUNK", "256")
    shape = (16, 16, 10)
    V = int(np.prod(shape))
    nm, na = (4, 3) if nc == 2 else (18, 8)

    def pinned(n):
        return torch.empty((V, 3, n), dtype=torch.float64, pin_memory=True).numpy()

    U0, E0 = state(oracle_port[nc], nc, shape, 17)
    lat = tcym.Lattice(ctx, nc, shape, tcym.FP32)
    lat.set_reunitarize_period(0)
    ref = tcym.Lattice(ctx, nc, shape, tcym.FP32)
    ref.set_reunitarize_period(0)
    Ua, Ea, Ub, Eb = pinned(nm), pinned(na), pinned(nm), pinned(na)
    Ua[:], Ea[:] = U0, E0
    Ur, Er = U0.copy(), E0.copy()
    for i, dt in enumerate([0.05, 0.05, 0.05, 0.03, 0.03]):
        if i < 4:
            lat.leapfrog_host(dt, Ua, Ea, Ua, Ea)  # in place
        else:
            lat.leapfrog_host(dt, Ua, Ea, Ub, Eb)  # new output arrays
            Ua, Ea = Ub, Eb
        ref.upload(Ur, Er)
        ref.leapfrog(dt, 1)
        Ur, Er = ref.download()
        assert np.array_equal(Ua, Ur) and np.array_equal(Ea, Er), i


def test_pinned_arrays_from_the_library(ctx, oracle_port):
    """tcym.pinned_empty (tcym_host_alloc): page-locked arrays take the captured-graph
    pipeline like any pinned memory and are freed with their last view."""
    import gc

    shape = (16, 16, 12)
    V = int(np.prod(shape))
    U0, E0 = state(oracle_port[3], 3, shape, 21)
    U, E = tcym.pinned_empty((V, 3, 18)), tcym.pinned_empty((V, 3, 8))
    assert U.flags.c_contiguous and U.flags.writeable and U.dtype == np.float64
    U[:], E[:] = U0, E0
    lat = tcym.Lattice(ctx, 3, shape, tcym.FP32)
    lat.set_reunitarize_period(0)
    for _ in range(2):
        lat.leapfrog_host(0.05, U, E, U, E)
    Us, Es = sequential(ctx, 3, shape, tcym.FP32, U0.copy(), E0.copy(), 0.05, 2)
    assert np.array_equal(U, Us) and np.array_equal(E, Es)
    view = U[:10]
    del U
    gc.collect()
    assert np.isfinite(view).all()  # the allocation lives while a view does
    del view, E
    gc.collect()
    assert tcym.pinned_empty((0,)).size == 0


@pytest.mark.parametrize("pinned", [False, True])
def test_host_step_two_copies_beyond_the_largest_pitch(ctx, oracle_port, monkeypatch, pinned):
    """Lattices whose half-state rows exceed the device's largest copy pitch (beyond
    ~200^3) move each chunk's two halves as two copies: forced here with a tiny limit."""
    monkeypatch.setenv("TCYM_HOST_STEP_MAX_PITCH", "4096")
    monkeypatch.setenv("TCYM_HOST_STEP_CHUNK", "128")
    shape = (16, 16, 8)
    V = int(np.prod(shape))
    U0, E0 = state(oracle_port[3], 3, shape, 25)
    if pinned:
        U, E = tcym.pinned_empty((V, 3, 18)), tcym.pinned_empty((V, 3, 8))
        U[:], E[:] = U0, E0
    else:
        U, E = U0.copy(), E0.copy()
    lat = tcym.Lattice(ctx, 3, shape, tcym.FP32)
    lat.set_reunitarize_period(0)
    for _ in range(2):
        lat.leapfrog_host(0.05, U, E, U, E)
    Us, Es = sequential(ctx, 3, shape, tcym.FP32, U0.copy(), E0.copy(), 0.05, 2)
    assert np.array_equal(U, Us) and np.array_equal(E, Es)
