"""ORACLE — test infrastructure, not product.

ctypes bindings for
  * ``liboracle.so``: the FP64 C restatement of the reference's hot path
    (tcym_oracle.c), built by ``make -C oracle`` on any host;
  * ``_ref/libref_su{2,3}.so``: the reference's own sources compiled in place
    (ref_wrap.cpp), present only where the reference tree was available.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs import this.
Arrays are the reference's AoS FP64 layouts:
  U: (V, 3, NM) doubles, NM = 4 (SU(2) quaternion) or 18 (SU(3), 9 complex, column-major)
  E: (V, 3, NA) doubles, NA = 3 or 8
with site index x + Nx*(y + Ny*z).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_dbl_p = ctypes.POINTER(ctypes.c_double)
_int_p = ctypes.POINTER(ctypes.c_int)

NM = {2: 4, 3: 18}
NA = {2: 3, 3: 8}
OBS_FIELDS = ("T00", "ELECTRIC", "MAGNETIC", "E0", "E1", "E2", "B0", "B1", "B2",
              "gauss_max", "gauss_rms", "unit_max", "unit_rms", "edotb_clover",
              "edotb_improved", "gauss_absmax")


def build(quiet: bool = True) -> None:
    """Compile liboracle.so (and the reference libs when the reference tree exists)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", HERE], check=True, stdout=out)
    ref_tree = os.environ.get("REFERENCE", "/root/reference")
    if os.path.isdir(ref_tree):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFERENCE={ref_tree}"], check=True, stdout=out)


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dbl_p)


def _n(shape):
    return (ctypes.c_int * 3)(*shape)


def empty_fields(nc: int, shape):
    V = int(np.prod(shape))
    return np.zeros((V, 3, NM[nc])), np.zeros((V, 3, NA[nc]))


class Port:
    """The C restatement for one gauge group (2 or 3)."""

    def __init__(self, nc: int):
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        self.lib = ctypes.CDLL(path)
        self.nc = nc
        self.g = f"orc_su{nc}_"
        L = self.lib
        f = self._f
        f("leapfrog").argtypes = [_int_p, _dbl_p, _dbl_p, ctypes.c_double, ctypes.c_int]
        f("update_e_only").argtypes = [_int_p, _dbl_p, _dbl_p, ctypes.c_double]
        f("update_u_only").argtypes = [_int_p, _dbl_p, _dbl_p, ctypes.c_double]
        f("langevin").argtypes = [_int_p, _dbl_p, _dbl_p, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int]
        f("flow").argtypes = [_int_p, _dbl_p, _dbl_p, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        f("flow").restype = ctypes.c_double
        f("flow_checkerboard").argtypes = [_int_p, _dbl_p, ctypes.c_double, ctypes.c_int]
        f("flow_checkerboard_cal").argtypes = [_int_p, _dbl_p, _dbl_p, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        f("flow_checkerboard_cal").restype = ctypes.c_double
        f("gauss_restore").argtypes = [_int_p, _dbl_p, _dbl_p, ctypes.c_double, ctypes.c_int]
        f("gauss_restore").restype = ctypes.c_int
        f("observables").argtypes = [_int_p, _dbl_p, _dbl_p, _dbl_p]
        f("edotb_clover").argtypes = [_int_p, _dbl_p, _dbl_p]
        f("edotb_clover").restype = ctypes.c_double
        f("edotb_improved").argtypes = [_int_p, _dbl_p, _dbl_p]
        f("edotb_improved").restype = ctypes.c_double
        f("set_zero").argtypes = [_int_p, _dbl_p, _dbl_p]
        f("gaussian_efield").argtypes = [_int_p, _dbl_p, ctypes.c_double, ctypes.c_uint64]
        f("gaussian_efield_step").argtypes = [_int_p, _dbl_p, ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64]
        f("thermalize").argtypes = [_int_p, _dbl_p, _dbl_p, ctypes.c_double, ctypes.c_uint64, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_int, _dbl_p, ctypes.c_int]
        f("thermalize").restype = ctypes.c_int
        f("ilog").argtypes = [ctypes.c_double, _dbl_p, _dbl_p]
        f("cool").argtypes = [_int_p, _dbl_p, ctypes.c_double, ctypes.c_int]
        f("block").argtypes = [_int_p, _dbl_p, _dbl_p]
        f("cool_blocked").argtypes = [_int_p, _dbl_p, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      _dbl_p]
        f("geodesic").argtypes = [_int_p, _dbl_p, _dbl_p, ctypes.c_double, _dbl_p, _dbl_p]
        f("cooled_delta_ncs").argtypes = [_int_p, _dbl_p, _dbl_p, ctypes.c_int]
        f("cooled_delta_ncs").restype = ctypes.c_double
        f("random_links").argtypes = [_int_p, _dbl_p, ctypes.c_double, ctypes.c_uint64]
        f("matrix_iexp").argtypes = [ctypes.c_double, _dbl_p, _dbl_p]
        f("retr_igen").argtypes = [_dbl_p, _dbl_p]
        f("adjoint").argtypes = [_dbl_p, _dbl_p, _dbl_p]
        f("inverse_adjoint").argtypes = [_dbl_p, _dbl_p, _dbl_p]
        L.orc_normal_c.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32,
                                   ctypes.c_uint32, ctypes.c_uint32]
        L.orc_normal_c.restype = ctypes.c_double
        L.orc_philox4x32.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3

    def _f(self, name):
        return getattr(self.lib, self.g + name)

    # lattice-level calls (arrays modified in place)
    def leapfrog(self, shape, U, E, dt, nsteps):
        self._f("leapfrog")(_n(shape), _p(U), _p(E), dt, nsteps)

    def update_e(self, shape, U, E, dt):
        self._f("update_e_only")(_n(shape), _p(U), _p(E), dt)

    def update_u(self, shape, U, E, dt):
        self._f("update_u_only")(_n(shape), _p(U), _p(E), dt)

    def langevin(self, shape, U, E, dt, gamma, T, seed, step0, nsteps):
        self._f("langevin")(_n(shape), _p(U), _p(E), dt, gamma, T, seed, step0, nsteps)

    def flow(self, shape, U, E, dtau, nsteps, calibrate=0):
        return self._f("flow")(_n(shape), _p(U), _p(E), dtau, nsteps, calibrate)

    def flow_checkerboard(self, shape, U, dtau, nsweeps):
        self._f("flow_checkerboard")(_n(shape), _p(U), dtau, nsweeps)

    def flow_checkerboard_cal(self, shape, U, E, dtau, nsweeps, calibrate=1):
        """Checkerboard sweeps with the cooled Delta N_CS (trapezoid, improved E.B by default)."""
        return self._f("flow_checkerboard_cal")(_n(shape), _p(U), _p(E), dtau, nsweeps, calibrate)

    def gauss_restore(self, shape, U, E, tol=1e-14, maxit=10000):
        return self._f("gauss_restore")(_n(shape), _p(U), _p(E), tol, maxit)

    def observables(self, shape, U, E):
        out = np.zeros(16)
        self._f("observables")(_n(shape), _p(U), _p(E), _p(out))
        return out

    def edotb_clover(self, shape, U, E):
        return self._f("edotb_clover")(_n(shape), _p(U), _p(E))

    def edotb_improved(self, shape, U, E):
        return self._f("edotb_improved")(_n(shape), _p(U), _p(E))

    def set_zero(self, shape, U, E):
        self._f("set_zero")(_n(shape), _p(U), _p(E))

    def gaussian_efield(self, shape, E, sigma, seed):
        self._f("gaussian_efield")(_n(shape), _p(E), sigma, seed)

    def gaussian_efield_step(self, shape, E, sigma, seed, step):
        self._f("gaussian_efield_step")(_n(shape), _p(E), sigma, seed, step)

    def thermalize(self, shape, U, E, beta, seed, rounds, max_time, dt=0.0375, every=20, cap=100000):
        """ThermalDynamics::Thermalize; returns the (records, 7) energy series."""
        series = np.zeros((cap, 7))
        n = self._f("thermalize")(_n(shape), _p(U), _p(E), beta, seed, rounds, max_time, dt, every, _p(series), cap)
        return series[:n].copy()

    def ilog(self, c, v):
        """A with exp(i c A^a t^a) = v (MatrixILog, principal branch)."""
        out = np.zeros(NA[self.nc])
        self._f("ilog")(c, _p(np.ascontiguousarray(v, dtype=np.float64)), _p(out))
        return out

    def cool(self, shape, U, sqrt_dctau, nsteps):
        self._f("cool")(_n(shape), _p(U), sqrt_dctau, nsteps)

    def block(self, shape, U):
        """Block(GaugeLinks**): the links of the lattice of half the extents."""
        Ub, _ = empty_fields(self.nc, tuple(k // 2 for k in shape))
        self._f("block")(_n(shape), _p(U), _p(Ub))
        return Ub

    def cool_blocked(self, shape, U, sqrt_dctau, nsteps, level, block_frequency):
        """Cooling::CoolNSave with `level` Blocks: the cooled links on shape / 2^level."""
        Uc, _ = empty_fields(self.nc, tuple(k >> level for k in shape))
        self._f("cool_blocked")(_n(shape), _p(U), sqrt_dctau, nsteps, level, block_frequency, _p(Uc))
        return Uc

    def geodesic(self, shape, Uold, Unew, c):
        Um, Em = empty_fields(self.nc, shape)
        self._f("geodesic")(_n(shape), _p(Uold), _p(Unew), c, _p(Um), _p(Em))
        return Um, Em

    def cooled_delta_ncs(self, shape, Uold, Unew, norder=1):
        return self._f("cooled_delta_ncs")(_n(shape), _p(Uold), _p(Unew), norder)

    def random_links(self, shape, U, sigma, seed):
        self._f("random_links")(_n(shape), _p(U), sigma, seed)

    # single objects
    def matrix_iexp(self, c, alpha):
        out = np.zeros(NM[self.nc])
        self._f("matrix_iexp")(c, _p(np.ascontiguousarray(alpha, dtype=np.float64)), _p(out))
        return out

    def retr_igen(self, v):
        out = np.zeros(NA[self.nc])
        self._f("retr_igen")(_p(np.ascontiguousarray(v, dtype=np.float64)), _p(out))
        return out

    def adjoint(self, v, e):
        out = np.zeros(NA[self.nc])
        self._f("adjoint")(_p(np.ascontiguousarray(v, dtype=np.float64)), _p(np.ascontiguousarray(e, dtype=np.float64)), _p(out))
        return out

    def inverse_adjoint(self, v, e):
        out = np.zeros(NA[self.nc])
        self._f("inverse_adjoint")(_p(np.ascontiguousarray(v, dtype=np.float64)), _p(np.ascontiguousarray(e, dtype=np.float64)), _p(out))
        return out

    def normal(self, seed, stream, step, site, mu, a):
        return self.lib.orc_normal_c(seed, stream, step, site, mu, a)

    def philox(self, ctr, key):
        c = (ctypes.c_uint32 * 4)(*ctr)
        k = (ctypes.c_uint32 * 2)(*key)
        o = (ctypes.c_uint32 * 4)()
        self.lib.orc_philox4x32(c, k, o)
        return list(o)


def ref_available(nc: int) -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", f"libref_su{nc}.so"))


def scipy_lapack():
    """(path, version) of the OpenBLAS build SciPy ships, whose LAPACK exports ZGEEV as
    ``scipy_zgeev_``, or None.  Setting TCYM_REF_LAPACK to the path makes the reference's
    SU(3) MatrixILog call that ZGEEV instead of the restatement in ``ref_wrap.cpp``."""
    try:
        import glob

        import scipy
    except ImportError:
        return None
    libs = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    for path in sorted(glob.glob(os.path.join(libs, "libscipy_openblas*.so"))):
        try:
            lib = ctypes.CDLL(path)
            lib.scipy_zgeev_
            get = lib.scipy_openblas_get_config
            get.restype = ctypes.c_char_p
            return path, get().decode().split(" DYNAMIC_ARCH")[0] + f" (SciPy {scipy.__version__})"
        except (OSError, AttributeError):
            continue
    return None


class Ref:
    """The reference's own sources, compiled in place (only where the reference tree exists).

    The reference keeps its lattice in globals, so one instance per group and one
    lattice at a time."""

    def __init__(self, nc: int):
        path = os.path.join(HERE, "_ref", f"libref_su{nc}.so")
        self.lib = L = ctypes.CDLL(path)
        self.nc = nc
        L.ref_init.argtypes = [ctypes.c_int] * 3
        L.ref_set.argtypes = [_dbl_p, _dbl_p]
        L.ref_get.argtypes = [_dbl_p, _dbl_p]
        L.ref_leapfrog.argtypes = [ctypes.c_double, ctypes.c_int]
        L.ref_update_e.argtypes = [ctypes.c_double]
        L.ref_update_u.argtypes = [ctypes.c_double]
        L.ref_langevin.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int]
        L.ref_flow.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.ref_flow.restype = ctypes.c_double
        L.ref_thermal_efield.argtypes = [ctypes.c_double, ctypes.c_uint64]
        L.ref_save_configuration.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint64]
        L.ref_cooling_init.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.ref_cooling_update.argtypes = [ctypes.c_int]
        L.ref_cooling_update.restype = ctypes.c_double
        L.ref_cooling_links.argtypes = [_dbl_p]
        L.ref_matrix_ilog.argtypes = [ctypes.c_double, _dbl_p, _dbl_p]
        L.ref_thermalize.argtypes = [ctypes.c_double, ctypes.c_uint64, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_char_p]
        L.ref_observables.argtypes = [_dbl_p]
        L.ref_matrix_iexp.argtypes = [ctypes.c_double, _dbl_p, _dbl_p]
        L.ref_retr_igen.argtypes = [_dbl_p, _dbl_p]
        L.ref_adjoint.argtypes = [_dbl_p, _dbl_p, _dbl_p]
        L.ref_inverse_adjoint.argtypes = [_dbl_p, _dbl_p, _dbl_p]
        self.shape = None

    def init(self, shape):
        self.shape = tuple(shape)
        self.lib.ref_init(*shape)

    def set(self, U, E):
        self.lib.ref_set(_p(U), _p(E))

    def get(self):
        U, E = empty_fields(self.nc, self.shape)
        self.lib.ref_get(_p(U), _p(E))
        return U, E

    def set_zero(self):
        self.lib.ref_set_zero()

    def leapfrog(self, dt, nsteps):
        self.lib.ref_leapfrog(dt, nsteps)

    def update_e(self, dt):
        self.lib.ref_update_e(dt)

    def update_u(self, dt):
        self.lib.ref_update_u(dt)

    def langevin(self, dt, T, seed, step0, nsteps):
        self.lib.ref_langevin(dt, T, seed, step0, nsteps)

    def flow(self, sqrt_dtau, nsteps, calibrate=0):
        return self.lib.ref_flow(sqrt_dtau, nsteps, calibrate)

    def gauss_restore(self):
        self.lib.ref_gauss_restore()

    def thermal_efield(self, beta, seed):
        self.lib.ref_thermal_efield(beta, seed)

    def observables(self):
        out = np.zeros(16)
        self.lib.ref_observables(_p(out))
        return out

    def save_configuration(self, outdir, ufname, efname, seed):
        """IO::SaveConfiguration; returns the two file paths."""
        import os
        self.lib.ref_save_configuration(str(outdir).encode(), ufname.encode(), efname.encode(), seed)
        return (os.path.join(str(outdir), f"{ufname}ID{seed}.txt"), os.path.join(str(outdir), f"{efname}ID{seed}.txt"))

    def cooling_init(self, blocking, max_steps, block_frequency, sqrt_dctau):
        self.lib.ref_cooling_init(blocking, max_steps, block_frequency, sqrt_dctau)

    def cooling_start(self):
        self.lib.ref_cooling_start()

    def cooling_update(self, measure):
        return self.lib.ref_cooling_update(measure)

    def cooling_links(self, blocking=0):
        """UOld of CoolingMethod (on the extents divided by 2^blocking)."""
        U, _ = empty_fields(self.nc, tuple(k >> blocking for k in self.shape))
        self.lib.ref_cooling_links(_p(U))
        return U

    def lapack_in_use(self) -> bool:
        """True when the reference's ZGEEV calls go to the library TCYM_REF_LAPACK names."""
        f = self.lib.ref_lapack_in_use
        f.restype = ctypes.c_int
        return bool(f())

    def matrix_ilog(self, c, v):
        out = np.zeros(NA[self.nc])
        self.lib.ref_matrix_ilog(c, _p(np.ascontiguousarray(v, dtype=np.float64)), _p(out))
        return out

    def thermalize(self, beta, seed, rounds, max_time, dtau, outdir):
        """ThermalDynamics::Thermalize; returns the (records, 7) series it writes to
        <outdir>/ThermalEnergyID<seed>.txt."""
        import os
        self.lib.ref_thermalize(beta, seed, rounds, max_time, dtau, str(outdir).encode())
        return np.loadtxt(os.path.join(str(outdir), f"ThermalEnergyID{seed}.txt"), ndmin=2)

    def matrix_iexp(self, c, alpha):
        out = np.zeros(NM[self.nc])
        self.lib.ref_matrix_iexp(c, _p(np.ascontiguousarray(alpha, dtype=np.float64)), _p(out))
        return out

    def retr_igen(self, v):
        out = np.zeros(NA[self.nc])
        self.lib.ref_retr_igen(_p(np.ascontiguousarray(v, dtype=np.float64)), _p(out))
        return out

    def adjoint(self, v, e):
        out = np.zeros(NA[self.nc])
        self.lib.ref_adjoint(_p(np.ascontiguousarray(v, dtype=np.float64)), _p(np.ascontiguousarray(e, dtype=np.float64)), _p(out))
        return out

    def inverse_adjoint(self, v, e):
        out = np.zeros(NA[self.nc])
        self.lib.ref_inverse_adjoint(_p(np.ascontiguousarray(v, dtype=np.float64)), _p(np.ascontiguousarray(e, dtype=np.float64)), _p(out))
        return out
