"""GB300-native real-time lattice Yang-Mills hot path (SU(2)/SU(3)).

Python mirror of the C ABI in ``include/tcym.h`` (libtcym.so, hand-written
sm_103a CUDA kernels).  Names follow the reference's C++ interface
(markmace/TopologicalCYMSolver): a :class:`Lattice` is the pair
GaugeLinks + ElectricFields; its methods are Dynamics::Update,
LangevinDynamics::Update, GradientFlow::StandardUpdate/CalibrationUpdate,
GaussLawRestoration::Restore, Observables::* and the Chern-Simons rate.

There is no CPU fallback: importing works anywhere, but creating a
:class:`Context` loads libtcym.so and needs a CUDA device; every failure is
raised as :class:`TcymError` with the library's message.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

__all__ = ["Context", "Lattice", "Observables", "TcymError", "FP32", "FP64", "FLOW_SIMULTANEOUS",
           "FLOW_CHECKERBOARD", "NCS_IMPROVED", "NCS_CLOVER", "library", "NM", "NA"]

FP64, FP32 = 0, 1
FLOW_SIMULTANEOUS, FLOW_CHECKERBOARD = 0, 1
NCS_IMPROVED, NCS_CLOVER = 1, 2  # E.B operator of calibrated flow
NM = {2: 4, 3: 18}   # doubles per link in the reference AoS layout
NA = {2: 3, 3: 8}    # algebra components

_ERRORS = {1: "invalid argument", 2: "device out of memory", 3: "CUDA error", 4: "non-finite state",
           5: "timeout", 6: "admission refused", 7: "invalid state"}


class TcymError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"tcym error {code} ({_ERRORS.get(code, '?')}): {msg}")
        self.code = code


class _Obs(ctypes.Structure):
    _fields_ = [("T00", ctypes.c_double), ("electric", ctypes.c_double), ("magnetic", ctypes.c_double),
                ("esqr", ctypes.c_double * 3), ("bsqr", ctypes.c_double * 3),
                ("gauss_max", ctypes.c_double), ("gauss_rms", ctypes.c_double), ("gauss_absmax", ctypes.c_double),
                ("unit_max", ctypes.c_double), ("unit_rms", ctypes.c_double),
                ("edotb", ctypes.c_double), ("ncs_dot", ctypes.c_double), ("ncs", ctypes.c_double),
                ("nonfinite", ctypes.c_int)]


@dataclass
class Observables:
    T00: float
    electric: float
    magnetic: float
    esqr: tuple
    bsqr: tuple
    gauss_max: float
    gauss_rms: float
    gauss_absmax: float
    unit_max: float
    unit_rms: float
    edotb: float
    ncs_dot: float
    ncs: float
    nonfinite: bool

    def as_oracle_vector(self) -> np.ndarray:
        """Same 16-slot order as the oracle's observables() output."""
        v = np.zeros(16)
        v[0], v[1], v[2] = self.T00, self.electric, self.magnetic
        v[3:6], v[6:9] = self.esqr, self.bsqr
        v[9], v[10], v[11], v[12], v[13] = self.gauss_max, self.gauss_rms, self.unit_max, self.unit_rms, self.edotb
        v[15] = self.gauss_absmax
        return v


class _Request(ctypes.Structure):
    _fields_ = [("nc", ctypes.c_int), ("L", ctypes.c_int), ("precision", ctypes.c_int), ("dynamics", ctypes.c_int),
                ("dt", ctypes.c_double), ("gamma", ctypes.c_double), ("T", ctypes.c_double), ("nsteps", ctypes.c_int),
                ("seed", ctypes.c_uint64)]


class _ServerInfo(ctypes.Structure):
    _fields_ = [("queued", ctypes.c_int), ("active", ctypes.c_int), ("completed", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("bytes_in_use", ctypes.c_size_t), ("link_updates", ctypes.c_double),
                ("preparing", ctypes.c_int), ("ticks", ctypes.c_uint64), ("prep_seconds", ctypes.c_double)]


_LIB = None
_dp = ctypes.POINTER(ctypes.c_double)
# tcym_tick: three doubles, two ints, padded to 32 bytes
TICK_DTYPE = np.dtype({"names": ["ms", "gap_ms", "link_updates", "active", "preparing"],
                       "formats": [np.float64, np.float64, np.float64, np.int32, np.int32],
                       "offsets": [0, 8, 16, 24, 28], "itemsize": 32})


def library() -> ctypes.CDLL:
    """Load libtcym.so (building it if the toolkit is present and it is missing or stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = os.environ.get("TCYM_LIBRARY", _build.LIB)  # another build of libtcym.so, if given
    if path == _build.LIB and (not os.path.exists(path) or os.environ.get("TCYM_REBUILD")):
        _build.build_library()
    L = ctypes.CDLL(path)
    c_void_pp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "tcym_version": ([], ctypes.c_int),
        "tcym_ctx_create": ([ctypes.c_int, c_void_pp], ctypes.c_int),
        "tcym_ctx_destroy": ([ctypes.c_void_p], ctypes.c_int),
        "tcym_last_error": ([ctypes.c_void_p], ctypes.c_char_p),
        "tcym_lattice_create": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int, c_void_pp], ctypes.c_int),
        "tcym_lattice_create_ex": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp,
                                    ctypes.c_int, c_void_pp], ctypes.c_int),
        "tcym_lattice_destroy": ([ctypes.c_void_p], ctypes.c_int),
        "tcym_lattice_bytes": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
        "tcym_lattice_upload": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
        "tcym_lattice_download": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
        "tcym_lattice_block": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
        "tcym_cooling_links": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
        "tcym_cooling_create_ex": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_void_p], ctypes.c_int),
        "tcym_leapfrog_host": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_void_p], ctypes.c_int),
        "tcym_lattice_copy": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
        "tcym_lattice_sync": ([ctypes.c_void_p], ctypes.c_int),
        "tcym_lattice_snapshot_bytes": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
        "tcym_lattice_snapshot": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t], ctypes.c_int),
        "tcym_lattice_restore": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t], ctypes.c_int),
        "tcym_lattice_snapshot_file": ([ctypes.c_void_p, ctypes.c_char_p], ctypes.c_int),
        "tcym_lattice_restore_file": ([ctypes.c_void_p, ctypes.c_char_p], ctypes.c_int),
        "tcym_lattice_noise_state": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
                                      ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "tcym_lattice_steps": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
        "tcym_lattice_stream": ([ctypes.c_void_p, c_void_pp], ctypes.c_int),
        "tcym_host_alloc": ([ctypes.c_size_t, c_void_pp], ctypes.c_int),
        "tcym_host_free": ([ctypes.c_void_p], ctypes.c_int),
        "tcym_set_zero": ([ctypes.c_void_p], ctypes.c_int),
        "tcym_gaussian_efield": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_uint64], ctypes.c_int),
        "tcym_write_configuration": ([ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p,
                                                          ctypes.c_char_p], ctypes.c_int),
        "tcym_read_configuration": ([ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p,
                                                         ctypes.c_char_p], ctypes.c_int),
        "tcym_lattice_save": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p], ctypes.c_int),
        "tcym_lattice_load": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p], ctypes.c_int),
        "tcym_lattice_tile": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
                              ctypes.c_int),
        "tcym_lattice_set_tile": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "tcym_cooling_create": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_double, c_void_pp], ctypes.c_int),
        "tcym_cooling_destroy": ([ctypes.c_void_p], ctypes.c_int),
        "tcym_cooling_start": ([ctypes.c_void_p], ctypes.c_int),
        "tcym_cooling_update": ([ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "tcym_cooling_delta_ncs": ([ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "tcym_cooling_total": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "tcym_thermalize": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_uint64, ctypes.c_int, ctypes.c_double,
                             ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                             ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "tcym_random_links": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_uint64], ctypes.c_int),
        "tcym_gauss_restore": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _dp],
                               ctypes.c_int),
        "tcym_leapfrog": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_int], ctypes.c_int),
        "tcym_update_e": ([ctypes.c_void_p, ctypes.c_double], ctypes.c_int),
        "tcym_update_u": ([ctypes.c_void_p, ctypes.c_double], ctypes.c_int),
        "tcym_langevin": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                           ctypes.c_uint64, ctypes.c_int], ctypes.c_int),
        "tcym_flow": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp], ctypes.c_int),
        "tcym_reunitarize": ([ctypes.c_void_p], ctypes.c_int),
        "tcym_set_reunitarize_period": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
        "tcym_observables": ([ctypes.c_void_p, ctypes.POINTER(_Obs)], ctypes.c_int),
        "tcym_edotb": ([ctypes.c_void_p, _dp], ctypes.c_int),
        "tcym_edotb_improved": ([ctypes.c_void_p, _dp], ctypes.c_int),
        "tcym_ncs_track": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
        "tcym_ncs_get": ([ctypes.c_void_p, _dp], ctypes.c_int),
        "tcym_ncs_reset": ([ctypes.c_void_p], ctypes.c_int),
        "tcym_ensemble_create": ([ctypes.c_void_p, c_void_pp], ctypes.c_int),
        "tcym_ensemble_destroy": ([ctypes.c_void_p], ctypes.c_int),
        "tcym_ensemble_add": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                               ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64], ctypes.c_int),
        "tcym_ensemble_remove": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
        "tcym_ensemble_set_persistent": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
        "tcym_ensemble_size": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "tcym_ensemble_step": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
        "tcym_ensemble_measure": ([ctypes.c_void_p, ctypes.c_int, _dp, _dp], ctypes.c_int),
        "tcym_server_create": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, c_void_pp],
                               ctypes.c_int),
        "tcym_server_destroy": ([ctypes.c_void_p], ctypes.c_int),
        "tcym_server_submit": ([ctypes.c_void_p, ctypes.POINTER(_Request), ctypes.POINTER(ctypes.c_uint64)],
                               ctypes.c_int),
        "tcym_server_status": ([ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int),
                                ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "tcym_server_wait": ([ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double], ctypes.c_int),
        "tcym_server_result": ([ctypes.c_void_p, ctypes.c_uint64, _dp, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                _dp], ctypes.c_int),
        "tcym_server_stats": ([ctypes.c_void_p, ctypes.POINTER(_ServerInfo)], ctypes.c_int),
        "tcym_server_ticks": ([ctypes.c_void_p, _dp, _dp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "tcym_server_tick_log": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)],
                                 ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _LIB = L
    return L


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.c_void_p)


class _PinnedBuffer:
    """Owns page-locked host memory from tcym_host_alloc; freed when the last array viewing it goes."""

    def __init__(self, nbytes: int):
        self.lib = library()
        p = ctypes.c_void_p()
        rc = self.lib.tcym_host_alloc(nbytes, ctypes.byref(p))
        if rc != 0:
            raise TcymError(rc, "tcym_host_alloc failed")
        self.ptr, self.nbytes = p.value, nbytes

    def __del__(self):
        if getattr(self, "ptr", None):
            self.lib.tcym_host_free(ctypes.c_void_p(self.ptr))
            self.ptr = None


def pinned_empty(shape, dtype=np.float64) -> np.ndarray:
    """A C-contiguous array in page-locked host memory (tcym_host_alloc): the host arrays
    of upload / download / leapfrog_host, whose copies then run asynchronously."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape))
    buf = _PinnedBuffer(max(1, n * dtype.itemsize))
    raw = (ctypes.c_char * buf.nbytes).from_address(buf.ptr)
    raw._owner = buf  # the ctypes array keeps the allocation alive; numpy keeps the ctypes array
    return np.frombuffer(raw, dtype=dtype, count=n).reshape(shape)


class Context:
    """A CUDA device opened by the library (tcym_ctx_create)."""

    def __init__(self, device: int = 0):
        self.lib = library()
        h = ctypes.c_void_p()
        rc = self.lib.tcym_ctx_create(device, ctypes.byref(h))
        if rc != 0:
            raise TcymError(rc, f"cannot open CUDA device {device}")
        self.h = h

    def check(self, rc: int) -> None:
        if rc != 0:
            msg = self.lib.tcym_last_error(self.h)
            raise TcymError(rc, msg.decode() if msg else "")

    def close(self) -> None:
        if self.h:
            self.lib.tcym_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Lattice:
    """GaugeLinks + ElectricFields on the device (LATTICE/GaugeLinks.cpp, LATTICE/ElectricFields.cpp)."""

    def __init__(self, ctx: Context, nc: int, shape, precision: int = FP64, spacing=None):
        self.ctx, self.lib, self.nc = ctx, ctx.lib, nc
        self.shape = tuple(int(n) for n in shape)
        self.precision = precision
        self.V = int(np.prod(self.shape))
        h = ctypes.c_void_p()
        if spacing is None:
            rc = self.lib.tcym_lattice_create(ctx.h, nc, *self.shape, precision, ctypes.byref(h))
        else:
            a = (ctypes.c_double * 3)(*spacing)
            rc = self.lib.tcym_lattice_create_ex(ctx.h, nc, *self.shape, a, precision, ctypes.byref(h))
        ctx.check(rc)
        self.h = h

    def close(self):
        if self.h:
            self.lib.tcym_lattice_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ state I/O
    def upload(self, U=None, E=None):
        self.ctx.check(self.lib.tcym_lattice_upload(self.h, _ptr(U), _ptr(E)))

    def download(self, U=None, E=None):
        """State as reference AoS FP64 arrays; pass preallocated (e.g. pinned) arrays to fill them."""
        U = np.empty((self.V, 3, NM[self.nc])) if U is None else U
        E = np.empty((self.V, 3, NA[self.nc])) if E is None else E
        self.ctx.check(self.lib.tcym_lattice_download(self.h, _ptr(U), _ptr(E)))
        return U, E

    def leapfrog_host(self, dt: float, U, E, U_out=None, E_out=None):
        """One leapfrog step of a state in host memory (reference AoS FP64 arrays):
        upload, step and download pipelined over z-ordered chunks; returns the new
        state (U_out, E_out, which may be U and E themselves)."""
        U_out = np.empty_like(U) if U_out is None else U_out
        E_out = np.empty_like(E) if E_out is None else E_out
        for a, n in ((U, NM[self.nc]), (E, NA[self.nc]), (U_out, NM[self.nc]), (E_out, NA[self.nc])):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != self.V * 3 * n:
                raise ValueError("leapfrog_host: C-contiguous float64 arrays of the reference AoS shapes expected")
        self.ctx.check(self.lib.tcym_leapfrog_host(self.h, dt, _ptr(U), _ptr(E), _ptr(U_out), _ptr(E_out)))
        return U_out, E_out

    def block_into(self, dst: "Lattice"):
        """Block(GaugeLinks**) + Block(ElectricFields**): dst (half the even extents, same
        group and precision) gets U'_mu(x) = U_mu(2x) U_mu(2x + mu), zero fields and
        twice the spacings."""
        self.ctx.check(self.lib.tcym_lattice_block(self.h, dst.h))

    def copy_from(self, other: "Lattice"):
        self.ctx.check(self.lib.tcym_lattice_copy(self.h, other.h))

    def nbytes(self) -> int:
        n = ctypes.c_size_t()
        self.ctx.check(self.lib.tcym_lattice_bytes(self.h, ctypes.byref(n)))
        return n.value

    def sync(self):
        self.ctx.check(self.lib.tcym_lattice_sync(self.h))

    def stream_handle(self) -> int:
        """cudaStream_t of the lattice (for torch.cuda.ExternalStream / event timing)."""
        p = ctypes.c_void_p()
        self.ctx.check(self.lib.tcym_lattice_stream(self.h, ctypes.byref(p)))
        return p.value or 0

    # ---------------------------------------------------- initial conditions
    def set_zero(self):
        self.ctx.check(self.lib.tcym_set_zero(self.h))

    def gaussian_efield(self, sigma: float, seed: int):
        self.ctx.check(self.lib.tcym_gaussian_efield(self.h, sigma, seed))

    def thermalize(self, beta: float, seed: int, rounds: int, max_time: float, dt: float = 0.0375,
                   every: int = 20, restore_tol: float = 0.0) -> np.ndarray:
        """ThermalDynamics::Thermalize; returns the (records, 7) ThermalEnergy series."""
        steps = 0
        while steps * dt < max_time:
            steps += 1
        cap = max(1, rounds * (steps // every if every > 0 else 0))
        series = np.zeros((cap, 7))
        n = ctypes.c_int(0)
        self.ctx.check(self.lib.tcym_thermalize(self.h, beta, seed, rounds, max_time, dt, restore_tol, every,
                                                series.ctypes.data_as(ctypes.c_void_p), cap, ctypes.byref(n)))
        return series[:n.value].copy()

    def tile(self):
        """(tx, ty) of the packed FP32 step's block tiling (autotuned on first use; tx 0: linear)."""
        tx, ty = ctypes.c_int(), ctypes.c_int()
        self.ctx.check(self.lib.tcym_lattice_tile(self.h, ctypes.byref(tx), ctypes.byref(ty)))
        return tx.value, ty.value

    def set_tile(self, tx: int, ty: int = 0):
        self.ctx.check(self.lib.tcym_lattice_set_tile(self.h, tx, ty))

    def save(self, ufile=None, efile=None):
        """The state to the reference's configuration text files (IO::SaveConfiguration)."""
        self.ctx.check(self.lib.tcym_lattice_save(self.h, _path(ufile), _path(efile)))

    def load(self, ufile=None, efile=None):
        """The state from the reference's configuration text files (IO::LoadConfiguration)."""
        self.ctx.check(self.lib.tcym_lattice_load(self.h, _path(ufile), _path(efile)))

    def random_links(self, sigma: float, seed: int):
        self.ctx.check(self.lib.tcym_random_links(self.h, sigma, seed))

    # ------------------------------------------------------------ snapshots
    def snapshot(self) -> bytearray:
        """Binary snapshot of the device state and its counters (tcym_lattice_snapshot)."""
        n = ctypes.c_size_t()
        self.ctx.check(self.lib.tcym_lattice_snapshot_bytes(self.h, ctypes.byref(n)))
        buf = bytearray(n.value)
        cbuf = (ctypes.c_char * n.value).from_buffer(buf)
        self.ctx.check(self.lib.tcym_lattice_snapshot(self.h, ctypes.addressof(cbuf), n.value))
        return buf

    def restore(self, buf) -> None:
        """State and counters from a snapshot of a lattice with the same group, precision and extents."""
        b = bytes(buf)
        self.ctx.check(self.lib.tcym_lattice_restore(self.h, b, len(b)))

    def snapshot_file(self, path) -> None:
        self.ctx.check(self.lib.tcym_lattice_snapshot_file(self.h, _path(path)))

    def restore_file(self, path) -> None:
        self.ctx.check(self.lib.tcym_lattice_restore_file(self.h, _path(path)))

    def noise_state(self):
        """(seed, next noise step, valid) of the last Langevin call."""
        seed, nxt, ok = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_int()
        self.ctx.check(self.lib.tcym_lattice_noise_state(self.h, ctypes.byref(seed), ctypes.byref(nxt),
                                                         ctypes.byref(ok)))
        return seed.value, nxt.value, bool(ok.value)

    def steps(self) -> int:
        n = ctypes.c_int64()
        self.ctx.check(self.lib.tcym_lattice_steps(self.h, ctypes.byref(n)))
        return n.value

    def gauss_restore(self, tol: float = 1e-14, maxit: int = 10000):
        it, mx = ctypes.c_int(), ctypes.c_double()
        self.ctx.check(self.lib.tcym_gauss_restore(self.h, tol, maxit, ctypes.byref(it), ctypes.byref(mx)))
        return it.value, mx.value

    # -------------------------------------------------------------- dynamics
    def leapfrog(self, dt: float, nsteps: int = 1):
        self.ctx.check(self.lib.tcym_leapfrog(self.h, dt, nsteps))

    def update_e(self, dt: float):
        self.ctx.check(self.lib.tcym_update_e(self.h, dt))

    def update_u(self, dt: float):
        self.ctx.check(self.lib.tcym_update_u(self.h, dt))

    def langevin(self, dt: float, gamma: float, T: float, seed: int, step0: int, nsteps: int = 1):
        self.ctx.check(self.lib.tcym_langevin(self.h, dt, gamma, T, seed, step0, nsteps))

    def flow(self, dtau: float, nsteps: int = 1, mode: int = FLOW_SIMULTANEOUS, calibrate: int = 0) -> float:
        """calibrate: 0 none, NCS_IMPROVED (the reference's NCsDot) or NCS_CLOVER; returns Delta N_CS."""
        d = ctypes.c_double()
        self.ctx.check(self.lib.tcym_flow(self.h, dtau, nsteps, mode, int(calibrate), ctypes.byref(d)))
        return d.value

    def reunitarize(self):
        self.ctx.check(self.lib.tcym_reunitarize(self.h))

    def set_reunitarize_period(self, period: int):
        self.ctx.check(self.lib.tcym_set_reunitarize_period(self.h, period))

    # ----------------------------------------------------------- observables
    def observables(self, allow_nonfinite: bool = False) -> Observables:
        o = _Obs()
        rc = self.lib.tcym_observables(self.h, ctypes.byref(o))
        if rc != 0 and not (allow_nonfinite and rc == 4):
            self.ctx.check(rc)
        return Observables(o.T00, o.electric, o.magnetic, tuple(o.esqr), tuple(o.bsqr), o.gauss_max, o.gauss_rms,
                           o.gauss_absmax, o.unit_max, o.unit_rms, o.edotb, o.ncs_dot, o.ncs, bool(o.nonfinite))

    def edotb(self) -> float:
        d = ctypes.c_double()
        self.ctx.check(self.lib.tcym_edotb(self.h, ctypes.byref(d)))
        return d.value

    def edotb_improved(self) -> float:
        d = ctypes.c_double()
        self.ctx.check(self.lib.tcym_edotb_improved(self.h, ctypes.byref(d)))
        return d.value

    def ncs_track(self, every: int = 1):
        self.ctx.check(self.lib.tcym_ncs_track(self.h, every))

    def ncs(self) -> float:
        d = ctypes.c_double()
        self.ctx.check(self.lib.tcym_ncs_get(self.h, ctypes.byref(d)))
        return d.value

    def ncs_reset(self):
        self.ctx.check(self.lib.tcym_ncs_reset(self.h))


def _path(p):
    return None if p is None else os.fsencode(p)


def write_configuration(nc: int, shape, U=None, E=None, ufile=None, efile=None) -> None:
    """Host arrays (the reference AoS layouts) to the reference's text files; no GPU needed."""
    rc = library().tcym_write_configuration(nc, *shape, _ptr(U) if U is not None else None,
                                            _ptr(E) if E is not None else None, _path(ufile), _path(efile))
    if rc:
        raise TcymError(rc, "tcym_write_configuration failed")


def read_configuration(nc: int, shape, ufile=None, efile=None):
    """The reference's text files to host arrays (U, E); no GPU needed."""
    V = int(np.prod(shape))
    U = np.zeros((V, 3, 4 if nc == 2 else 18)) if ufile else None
    E = np.zeros((V, 3, 3 if nc == 2 else 8)) if efile else None
    rc = library().tcym_read_configuration(nc, *shape, _ptr(U) if U is not None else None,
                                           _ptr(E) if E is not None else None, _path(ufile), _path(efile))
    if rc:
        raise TcymError(rc, "tcym_read_configuration: unreadable or incomplete files")
    return U, E


class Cooling:
    """ChernSimonsNumber::CoolingMethod (tcym_cooling_*): cooled copies of a lattice's
    links (blocked blocking_level times, after steps block_frequency 8^b) and the
    cooled real-time Delta N_CS between them."""

    def __init__(self, lat: "Lattice", max_steps: int = 128, sqrt_dctau: float = 0.125 ** 0.5,
                 blocking_level: int = 0, block_frequency: int = 0):
        self.lat, self.ctx, self.lib = lat, lat.ctx, lat.lib
        h = ctypes.c_void_p()
        self.ctx.check(self.lib.tcym_cooling_create_ex(lat.h, max_steps, sqrt_dctau, blocking_level, block_frequency,
                                                       ctypes.byref(h)))
        self.h = h
        self.level = blocking_level

    def start(self):
        self.ctx.check(self.lib.tcym_cooling_start(self.h))

    def update(self, measure: bool = True) -> float:
        d = ctypes.c_double()
        self.ctx.check(self.lib.tcym_cooling_update(self.h, int(measure), ctypes.byref(d)))
        return d.value

    def delta_ncs(self, norder: int = 1) -> float:
        d = ctypes.c_double()
        self.ctx.check(self.lib.tcym_cooling_delta_ncs(self.h, norder, ctypes.byref(d)))
        return d.value

    def links(self):
        """The latest cooled links (AoS FP64, on the lattice's extents / 2^blocking_level)."""
        V = self.lat.V >> (3 * self.level)
        U = np.empty((V, 3, NM[self.lat.nc]))
        self.ctx.check(self.lib.tcym_cooling_links(self.h, _ptr(U)))
        return U

    def total(self) -> float:
        d = ctypes.c_double()
        self.ctx.check(self.lib.tcym_cooling_total(self.h, ctypes.byref(d)))
        return d.value

    def close(self):
        if self.h:
            self.lib.tcym_cooling_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


DYN_LEAPFROG, DYN_LANGEVIN = 0, 1


class Ensemble:
    """Independent lattices advanced together (tcym_ensemble_*): one batched,
    graph-captured launch per storage format and step."""

    def __init__(self, ctx: Context):
        self.ctx, self.lib = ctx, ctx.lib
        h = ctypes.c_void_p()
        ctx.check(self.lib.tcym_ensemble_create(ctx.h, ctypes.byref(h)))
        self.h = h
        self.members = []

    def add(self, lat: Lattice, dt: float, dynamics: int = DYN_LEAPFROG, gamma: float = 0.0, T: float = 0.0,
            seed: int = 0, step0: int = 0):
        self.ctx.check(self.lib.tcym_ensemble_add(self.h, lat.h, dynamics, dt, gamma, T, seed, step0))
        self.members.append(lat)

    def set_persistent(self, group_blocks: int = 0):
        """K-step persistent launches (group_blocks >= 0, members in groups of at least that
        many blocks; 0: one group) or one launch per step (group_blocks < 0)."""
        self.ctx.check(self.lib.tcym_ensemble_set_persistent(self.h, group_blocks))

    def remove(self, lat: Lattice):
        self.ctx.check(self.lib.tcym_ensemble_remove(self.h, lat.h))
        self.members.remove(lat)

    def __len__(self):
        return len(self.members)

    def step(self, nsteps: int):
        self.ctx.check(self.lib.tcym_ensemble_step(self.h, nsteps))

    def measure(self, ncs_stride: int = 0):
        """(E.B, N_CS) arrays in member order; ncs_stride > 0 advances each member's N_CS."""
        n = len(self.members)
        edb, ncs = np.zeros(n), np.zeros(n)
        self.ctx.check(self.lib.tcym_ensemble_measure(self.h, ncs_stride, edb.ctypes.data_as(_dp),
                                                      ncs.ctypes.data_as(_dp)))
        return edb, ncs

    def close(self):
        if self.h:
            self.lib.tcym_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


class Server:
    """Continuous-batching request loop (tcym_server_*): requests are admitted by
    device-memory footprint, advanced together and retired as they finish."""

    def __init__(self, ctx: Context, hbm_budget_bytes: int, max_active: int = 512, stride: int = 20):
        self.ctx, self.lib = ctx, ctx.lib
        h = ctypes.c_void_p()
        ctx.check(self.lib.tcym_server_create(ctx.h, hbm_budget_bytes, max_active, stride, ctypes.byref(h)))
        self.h = h

    def submit(self, nc: int, L: int, T: float, nsteps: int, dynamics: int = DYN_LEAPFROG, dt: float = 0.05,
               gamma: float = 1.0, precision: int = FP32, seed: int = 0) -> int:
        r = _Request(nc, L, precision, dynamics, dt, gamma, T, nsteps, seed)
        i = ctypes.c_uint64()
        self.ctx.check(self.lib.tcym_server_submit(self.h, ctypes.byref(r), ctypes.byref(i)))
        return i.value

    def status(self, rid: int):
        s, n = ctypes.c_int(), ctypes.c_int()
        self.ctx.check(self.lib.tcym_server_status(self.h, rid, ctypes.byref(s), ctypes.byref(n)))
        return s.value, n.value

    def wait(self, rid: int, timeout_s: float = 600.0) -> int:
        """Status code of the bounded wait (0 = done, 5 = timed out, else the request's error)."""
        return self.lib.tcym_server_wait(self.h, rid, timeout_s)

    def result(self, rid: int):
        """(series (n, 2) of (steps, N_CS), latency in s, status code)."""
        n, lat = ctypes.c_int(), ctypes.c_double()
        rc = self.lib.tcym_server_result(self.h, rid, None, 0, ctypes.byref(n), ctypes.byref(lat))
        if rc not in (0, 4) and n.value == 0 and lat.value == 0.0:
            self.ctx.check(rc)
        buf = np.zeros((max(n.value, 1), 2))
        rc = self.lib.tcym_server_result(self.h, rid, buf.ctypes.data_as(_dp), n.value, ctypes.byref(n),
                                         ctypes.byref(lat))
        return buf[: n.value], lat.value, rc

    def stats(self) -> dict:
        s = _ServerInfo()
        self.ctx.check(self.lib.tcym_server_stats(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in _ServerInfo._fields_}

    def ticks(self, capacity: int = 8192):
        """(ms, preparing) arrays of the last ticks, oldest first."""
        ms, prep, n = np.zeros(capacity), np.zeros(capacity), ctypes.c_int()
        self.ctx.check(self.lib.tcym_server_ticks(self.h, ms.ctypes.data_as(_dp), prep.ctypes.data_as(_dp), capacity,
                                                  ctypes.byref(n)))
        return ms[: n.value], prep[: n.value]

    def tick_log(self, capacity: int = 8192) -> np.ndarray:
        """The last ticks as a structured array (ms, gap_ms, link_updates, active, preparing),
        oldest first (tcym_tick)."""
        rec = np.zeros(capacity, dtype=TICK_DTYPE)
        n = ctypes.c_int()
        self.ctx.check(self.lib.tcym_server_tick_log(self.h, rec.ctypes.data_as(ctypes.c_void_p), capacity,
                                                     ctypes.byref(n)))
        return rec[: n.value]

    def close(self):
        if self.h:
            self.lib.tcym_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
