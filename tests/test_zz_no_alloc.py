"""The allocation-free Gauss restore against the allocating one.

tcym_gauss_restore_noalloc serves callers that cannot let a library allocate
device memory (their allocator owns the GPU, or their loop must never pay for
cudaMalloc/cudaFree).  Here the test plays such a caller: it owns the AoS FP64
buffers on the device (allocated with torch), calls the entry point through the
C ABI twice in a row (SU(3), then SU(2), sharing the library's one scratch
array), and compares each result with tcym_gauss_restore on a lattice built
from the same input, within the FP64 device tolerance of the parity tests.

This file sorts last so that a run stopping at its first failure has already
run every other test.
"""
import ctypes

import numpy as np
import pytest

import oracle
import topologicalcymsolver_gb300 as tcym

pytestmark = pytest.mark.gpu

TOL = 1e-10  # FP64 device path, as tests/test_gpu_parity.py


def _bind(lib):
    f = lib.tcym_gauss_restore_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                  ctypes.POINTER(ctypes.c_double), ctypes.c_char_p, ctypes.c_size_t]
    f.restype = ctypes.c_int
    return f


def _restore_noalloc(f, nc, shape, U_dev, E_dev, stream):
    it, mx = ctypes.c_int(-1), ctypes.c_double(-1.0)
    err = ctypes.create_string_buffer(512)
    rc = f(nc, *shape, ctypes.c_void_p(U_dev), ctypes.c_void_p(E_dev), 1e-14, 10000, ctypes.c_void_p(stream),
           ctypes.byref(it), ctypes.byref(mx), err, 512)
    return rc, it.value, mx.value, err.value.decode()


def _input(nc, shape, seed):
    P = oracle.Port(nc)
    U, E = oracle.empty_fields(nc, shape)
    P.random_links(shape, U, 0.6, seed)
    P.gaussian_efield(shape, E, 0.7, seed + 1)
    return P, U, E


def test_noalloc_restore_matches_allocating_restore_twice(ctx):
    torch = pytest.importorskip("torch")
    oracle.build()
    f = _bind(tcym.library())
    for nc, shape, seed in ((3, (6, 6, 6), 71), (2, (8, 6, 10), 73)):
        P, U, E = _input(nc, shape, seed)
        # the existing entry point
        lat = tcym.Lattice(ctx, nc, shape, tcym.FP64)
        lat.upload(U, E)
        it_ref, mx_ref = lat.gauss_restore(1e-14, 10000)
        _, E_ref = lat.download()
        lat.close()
        # the caller's own device buffers
        dev = torch.device("cuda", 0)
        U_d = torch.from_numpy(U).to(dev)
        E_d = torch.from_numpy(E).to(dev)
        torch.cuda.synchronize()
        stream = torch.cuda.current_stream(dev).cuda_stream
        free_before = torch.cuda.mem_get_info(dev)[0]
        rc, it, mx, msg = _restore_noalloc(f, nc, shape, U_d.data_ptr(), E_d.data_ptr(), stream)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(dev)[0]
        assert rc == 0, msg
        E_out = E_d.cpu().numpy()
        assert abs(it - it_ref) <= 1
        rel = np.abs(E_out - E_ref).max() / np.abs(E_ref).max()
        assert rel < TOL, rel
        assert np.array_equal(U_d.cpu().numpy(), U)  # links are read only
        o = P.observables(shape, U, E_out)
        assert o[9] <= 1e-13 and mx <= 1e-14 and mx_ref <= 1e-14
        if nc == 2:  # second call: the scratch is set up; no device memory was taken
            assert free_after == free_before


def test_noalloc_reports_a_nan_in_the_field(ctx):
    """One NaN in E: the maxima drop it (fmax), the sums do not; the call must
    return TCYM_ERR_NONFINITE instead of a converged restore."""
    torch = pytest.importorskip("torch")
    oracle.build()
    f = _bind(tcym.library())
    for nc, shape, seed in ((3, (6, 6, 6), 75), (2, (8, 6, 10), 77)):
        _, U, E = _input(nc, shape, seed)
        E[17, 1, 2] = np.nan
        dev = torch.device("cuda", 0)
        U_d = torch.from_numpy(U).to(dev)
        E_d = torch.from_numpy(E).to(dev)
        torch.cuda.synchronize()
        stream = torch.cuda.current_stream(dev).cuda_stream
        rc, it, _, msg = _restore_noalloc(f, nc, shape, U_d.data_ptr(), E_d.data_ptr(), stream)
        torch.cuda.synchronize()
        assert rc == 4, (rc, msg)
        assert it == 0 and "NaN" in msg


def test_noalloc_rejects_lattices_beyond_the_scratch(ctx):
    f = _bind(tcym.library())
    # 52^3 SU(3) sites need 8 * 140608 doubles > 1,036,272: rejected before touching the buffers
    rc, _, _, msg = _restore_noalloc(f, 3, (52, 52, 52), 0x1000, 0x2000, 0)
    assert rc == 1 and "too large" in msg
    rc, _, _, msg = _restore_noalloc(f, 2, (71, 71, 71), 0x1000, 0x2000, 0)
    assert rc == 1 and "too large" in msg
