"""ctypes helper for libtcym_hostcheck.so: the per-site device code of the
kernels, instantiated for the host (test-only).  A HostLattice holds host
buffers in the exact device storage layout of one format."""
import ctypes

import numpy as np

from topologicalcymsolver_gb300 import build as _build

FMT = {(2, "f32"): 0, (2, "f64"): 1, (3, "f32"): 2, (3, "f64"): 3}
LINK_BYTES = {0: 16, 1: 32, 2: 48, 3: 144}
FIELD_BYTES = {0: 12, 1: 24, 2: 32, 3: 64}
NM = {2: 4, 3: 18}
NA = {2: 3, 3: 8}

_L = None
_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)


def load():
    global _L
    if _L is None:
        _build.build_hostcheck()
        L = ctypes.CDLL(_build.HOSTCHECK)
        ip = ctypes.POINTER(ctypes.c_int)
        L.hc_from_aos.argtypes = [ctypes.c_int, ip, _vp, _vp, _vp, _vp]
        L.hc_to_aos.argtypes = [ctypes.c_int, ip, _vp, _vp, _vp, _vp]
        L.hc_step.argtypes = [ctypes.c_int, ip, _vp, _vp, _vp, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                              ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int]
        L.hc_flow_cb.argtypes = [ctypes.c_int, ip, _vp, ctypes.c_double, ctypes.c_int]
        L.hc_observables.argtypes = [ctypes.c_int, ip, _vp, _vp, ctypes.c_int, _vp]
        L.hc_edotb_pair.argtypes = [ctypes.c_int, ip, _vp, _vp, _vp]
        L.hc_gauss_restore.argtypes = [ctypes.c_int, ip, _vp, _vp, ctypes.c_double, ctypes.c_int]
        L.hc_reunitarize.argtypes = [ctypes.c_int, ip, _vp]
        L.hc_block.argtypes = [ctypes.c_int, ip, _vp, _vp]
        L.hc_from_aos_range.argtypes = [ctypes.c_int, ip, _vp, _vp, _vp, _vp, ctypes.c_int64, ctypes.c_int64]
        L.hc_step_range.argtypes = [ctypes.c_int, ip, _vp, _vp, _vp, ctypes.c_double, ctypes.c_int64, ctypes.c_int64]
        L.hc_init.argtypes = [ctypes.c_int, ip, _vp, _vp, ctypes.c_int, ctypes.c_double, ctypes.c_uint64]
        L.hc_iexp.argtypes = [ctypes.c_int, ctypes.c_double, _vp, _vp]
        L.hc_ilog.argtypes = [ctypes.c_int, ctypes.c_double, _vp, _vp]
        L.hc_geodesic.argtypes = [ctypes.c_int, ip, _vp, _vp, ctypes.c_double, _vp, _vp]
        L.hc_normal.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                ctypes.c_uint32, ctypes.c_int]
        L.hc_normal.restype = ctypes.c_double
        L.hc_pipeline_schedule.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _vp, ctypes.c_int64, _vp,
                                           _vp, ctypes.c_int64]
        L.hc_pipeline_schedule.restype = ctypes.c_int64
        _L = L
    return _L


def _p(a):
    return a.ctypes.data_as(_vp)


class HostLattice:
    """Host arrays in the device layout of format (nc, prec), ping-pong links like the library."""

    def __init__(self, nc, prec, shape):
        self.L = load()
        self.nc, self.fmt = nc, FMT[(nc, prec)]
        self.shape = tuple(shape)
        self.n = (ctypes.c_int * 3)(*shape)
        self.V = int(np.prod(shape))
        # the FP32 formats store site pairs, padded to an even site count
        stored = 2 * ((self.V + 1) // 2) if prec == "f32" else self.V
        self.U = [np.zeros(3 * LINK_BYTES[self.fmt] * stored, np.uint8) for _ in range(2)]
        self.E = np.zeros(3 * FIELD_BYTES[self.fmt] * stored, np.uint8)
        self.cur = 0
        self.pairs = 1  # 0: the per-site step; 1 + tx: the paired step with block tiling tx (0: linear)

    def upload(self, U=None, E=None):
        self.L.hc_from_aos(self.fmt, self.n, None if U is None else _p(U), None if E is None else _p(E),
                           _p(self.U[self.cur]), _p(self.E))

    def download(self):
        U = np.zeros((self.V, 3, NM[self.nc]))
        E = np.zeros((self.V, 3, NA[self.nc]))
        self.L.hc_to_aos(self.fmt, self.n, _p(self.U[self.cur]), _p(self.E), _p(U), _p(E))
        return U, E

    def step(self, mode, dt, gamma=0.0, T=0.0, seed=0, step=0, do_e=True, do_u=True):
        if do_e and do_u:
            self.L.hc_step(self.fmt, self.n, _p(self.U[self.cur]), _p(self.U[1 - self.cur]), _p(self.E), mode, dt,
                           gamma, T, seed, step, 1, 1, self.pairs)
            self.cur ^= 1
        else:
            self.L.hc_step(self.fmt, self.n, _p(self.U[self.cur]), _p(self.U[self.cur]), _p(self.E), mode, dt, gamma,
                           T, seed, step, int(do_e), int(do_u), self.pairs)

    def leapfrog(self, dt, nsteps):
        for _ in range(nsteps):
            self.step(0, dt)

    def langevin(self, dt, gamma, T, seed, step0, nsteps):
        for i in range(nsteps):
            self.step(1, dt, gamma, T, seed, step0 + i)

    def flow(self, dtau, nsteps):
        for _ in range(nsteps):
            self.step(2, dtau)

    def flow_checkerboard(self, dtau, nsweeps):
        self.L.hc_flow_cb(self.fmt, self.n, _p(self.U[self.cur]), dtau, nsweeps)

    def observables(self, mask=15):
        out = np.zeros(16)
        self.L.hc_observables(self.fmt, self.n, _p(self.U[self.cur]), _p(self.E), mask, _p(out))
        return out

    def edotb_pair(self):
        """The N_CS sample through the paired code, or None where the storage is not paired."""
        out = np.zeros(16)
        ok = self.L.hc_edotb_pair(self.fmt, self.n, _p(self.U[self.cur]), _p(self.E), _p(out))
        return out if ok else None

    def gauss_restore(self, tol=1e-14, maxit=10000):
        return self.L.hc_gauss_restore(self.fmt, self.n, _p(self.U[self.cur]), _p(self.E), tol, maxit)

    def reunitarize(self):
        self.L.hc_reunitarize(self.fmt, self.n, _p(self.U[self.cur]))

    def poison(self):
        """Every stored value NaN (so that reading anything not written since shows)."""
        for a in (*self.U, self.E):
            if a.dtype.kind == "f":
                a[...] = np.nan
            else:
                a.view(np.float32 if self.fmt in (0, 2) else np.float64)[...] = np.nan

    def from_aos_range(self, U, E, s0, count):
        self.L.hc_from_aos_range(self.fmt, self.n, _p(U), _p(E), _p(self.U[self.cur]), _p(self.E), s0, count)

    def step_range(self, dt, i0, i1):
        """One leapfrog step of storage indices [i0, i1), new links into the other buffer."""
        self.L.hc_step_range(self.fmt, self.n, _p(self.U[self.cur]), _p(self.U[1 - self.cur]), _p(self.E), dt, i0, i1)

    def block_into(self, other):
        """Block (site_block) of this lattice's links into `other` (half the extents)."""
        self.L.hc_block(self.fmt, self.n, _p(self.U[self.cur]), _p(other.U[other.cur]))

    def init(self, what, sigma=0.0, seed=0):
        self.L.hc_init(self.fmt, self.n, _p(self.U[self.cur]), _p(self.E), what, sigma, seed)

    def geodesic(self, old, new, c):
        """UMid, EMid (into this lattice) of the geodesic from old's links to new's."""
        self.L.hc_geodesic(self.fmt, self.n, _p(old.U[old.cur]), _p(new.U[new.cur]), c, _p(self.U[self.cur]),
                           _p(self.E))


def iexp(nc, prec, c, alpha):
    L = load()
    out = np.zeros(NM[nc])
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    L.hc_iexp(FMT[(nc, prec)], c, _p(a), _p(out))
    return out


def ilog(nc, prec, c, v):
    L = load()
    out = np.zeros(NA[nc])
    L.hc_ilog(FMT[(nc, prec)], c, _p(np.ascontiguousarray(v, dtype=np.float64)), _p(out))
    return out


def normal(seed, stream, step, site, mu, a, single=False):
    return load().hc_normal(seed, stream, step, site, mu, a, int(single))


def pipeline_schedule(N, P, C):
    """(bounds, [(kind, chunk)]) of the host-resident step's pipeline (0 upload, 1 step)."""
    L = load()
    cap = 4 * ((N + 127) // 128) + 16
    bounds = np.zeros(cap, np.int64)
    kinds, chunks = np.zeros(2 * cap, np.int32), np.zeros(2 * cap, np.int64)
    n = L.hc_pipeline_schedule(N, P, C, _p(bounds), cap, _p(kinds), _p(chunks), 2 * cap)
    assert n <= 2 * cap
    nchunks = n // 2
    return bounds[:nchunks + 1].tolist(), list(zip(kinds[:n].tolist(), chunks[:n].tolist()))
