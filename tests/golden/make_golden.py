"""Generate the golden fixtures of tests/golden/ from the reference's own code.

Runs the reference's hot-path sources compiled in place (oracle/_ref, built by
``make -C oracle ref`` from the reference tree) on small seeded inputs and
stores inputs and outputs as .npz.  The reference tree is needed only to
regenerate; the fixtures are committed and the tests read them anywhere.

Inputs are built with the oracle's Philox generators (the same streams the
CUDA library draws); every output below is produced by the reference itself:
  ref_states_su{2,3}.npz   (4,5,6) lattice: leapfrog 1/10/100 steps (dt 0.05),
                           Langevin 10 steps (dt 0.02, gamma 1, T 0.6, seed 3),
                           gradient flow 10 steps (dtau 0.02, CalibrationUpdate),
                           Gauss restore, and the observables of each state
  ref_group_su{2,3}.npz    MatrixIExp, ReTrIGenU, (Inverse)AdjointMultiplication
  ref_leapfrog_su2_16.npz  SU(2) 16^3 leapfrog series: U = 1, E ~ N(0, 1/2)
                           (seed 1) Gauss-restored by the reference, 1000 leapfrog
                           steps at dt 0.05, observables every 10 steps
  ref_thermalize_su{2,3}.npz  ThermalDynamics::Thermalize(2, 0.75) on a (4,4,6)
                           lattice from U = 1, beta 2, seed 7, dTau 0.0375 (20
                           steps a round): final U, E and the ThermalEnergy file
                           (every 20 steps; the reference writes 6 digits)
  ref_config_su{2,3}_U.txt, ref_config_su{2,3}_E.txt, ref_config_su{2,3}.npz
                           IO::SaveConfiguration of a random (3,4,5) state (links
                           seed 21, sigma 0.6; fields seed 22, sigma 0.7): the
                           reference's text files and the arrays they hold
  ref_cooling_su2.npz      ChernSimonsNumber::CoolingMethod, SU(2) (6,6,6): a
                           random-link state (seed 3, sigma 0.5; E seed 4, 0.7,
                           restored); Start, then 3 x (20 leapfrog steps at dt
                           0.05, Update(1)) with 16 cooling steps of sqrt_dctau
                           sqrt(0.02): the cumulative DeltaNCsCoolRealTime after
                           each update and the cooled links
  ref_cooling_su3.npz      the same for SU(3) at blocking levels 0 (6^3) and 1
                           (8^3), the reference's MatrixILog calling LAPACK's ZGEEV
                           from the OpenBLAS that SciPy ships (key "zgeev" names it)
  ref_cooling_su2_96.npz   the SU(2) 96^3 gradient-flow cooling run: U = 1, E ~
                           N(0, 1/2) (seed 4) restored by the reference, 2000
                           leapfrog steps of dt 0.05 by the reference, then 500
                           sweeps of dtau 0.02 with the cooled N_CS along the flow
                           (improved E.B, trapezoid): simultaneous sweeps by the
                           reference itself (GradientFlow::CalibrationUpdate) and
                           checkerboarded sweeps by the oracle's restatement (the
                           reference has none); (T00, ELECTRIC, MAGNETIC, Delta
                           N_CS so far) every 10 sweeps, the start's observables and
                           a few links and fields of the start as its fingerprint

  python tests/golden/make_golden.py [generator ...]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

SHAPE = (4, 5, 6)


def states(nc):
    P, R = oracle.Port(nc), oracle.Ref(nc)
    U0, E0 = oracle.empty_fields(nc, SHAPE)
    P.random_links(SHAPE, U0, 0.6, 101 + nc)
    P.gaussian_efield(SHAPE, E0, 0.7, 201 + nc)
    R.init(SHAPE)
    out = {"U0": U0, "E0": E0, "shape": np.array(SHAPE)}

    def obs(tag):
        out["obs_" + tag] = R.observables()

    R.set(U0, E0)
    obs("0")
    R.leapfrog(0.05, 1)
    out["U_lf1"], out["E_lf1"] = R.get()
    obs("lf1")
    R.leapfrog(0.05, 9)
    out["U_lf10"], out["E_lf10"] = R.get()
    obs("lf10")
    R.leapfrog(0.05, 90)
    out["U_lf100"], out["E_lf100"] = R.get()
    obs("lf100")

    R.set(U0, E0)
    R.langevin(0.02, 0.6, 3, 0, 10)
    out["U_lv10"], out["E_lv10"] = R.get()
    obs("lv10")

    R.set(U0, E0)
    out["dncs_fl10"] = np.array(R.flow(np.sqrt(0.02), 10, 1))
    out["U_fl10"], out["E_fl10"] = R.get()
    obs("fl10")

    R.set(U0, E0)
    R.gauss_restore()
    out["U_gr"], out["E_gr"] = R.get()
    obs("gr")
    np.savez_compressed(os.path.join(HERE, f"ref_states_su{nc}.npz"), **out)


def group(nc):
    R = oracle.Ref(nc)
    rng = np.random.default_rng(7 + nc)
    na = oracle.NA[nc]
    n = 12
    alpha = rng.normal(size=(n, na)) * np.repeat([1e-4, 0.1, 1.0, 4.0], 3)[:, None]
    c = rng.normal(size=n)
    exps = np.array([R.matrix_iexp(c[i], alpha[i]) for i in range(n)])
    e = rng.normal(size=(n, na))
    proj = np.array([R.retr_igen(exps[i] * 1.1) for i in range(n)])
    adj = np.array([R.adjoint(exps[i], e[i]) for i in range(n)])
    iadj = np.array([R.inverse_adjoint(exps[i], e[i]) for i in range(n)])
    np.savez_compressed(os.path.join(HERE, f"ref_group_su{nc}.npz"), alpha=alpha, c=c, exp=exps, e=e, proj=proj,
                        adj=adj, iadj=iadj)


def leapfrog_series_su2_16():
    R = oracle.Ref(2)
    shape = (16, 16, 16)
    R.init(shape)
    R.set_zero()
    R.thermal_efield(2.0, 1)  # E = N(0,1)/sqrt(2) then Restore (ThermalDynamics.cpp:205-226)
    U, E = R.get()
    series = [R.observables()]
    for _ in range(100):
        R.leapfrog(0.05, 10)
        series.append(R.observables())
    np.savez_compressed(os.path.join(HERE, "ref_leapfrog_su2_16.npz"), E_ic=E, series=np.array(series), dt=0.05,
                        every=10)


def thermalize(nc):
    import tempfile
    R = oracle.Ref(nc)
    shape = (4, 4, 6)
    R.init(shape)
    R.set_zero()
    with tempfile.TemporaryDirectory() as d:
        series = R.thermalize(2.0, 7, 2, 0.75, 0.0375, d)
    U, E = R.get()
    np.savez_compressed(os.path.join(HERE, f"ref_thermalize_su{nc}.npz"), U=U, E=E, series=series,
                        shape=np.array(shape), beta=2.0, seed=7, rounds=2, max_time=0.75, dtau=0.0375)


def configuration(nc):
    import shutil
    import tempfile
    P, R = oracle.Port(nc), oracle.Ref(nc)
    shape = (3, 4, 5)
    U, E = oracle.empty_fields(nc, shape)
    P.random_links(shape, U, 0.6, 21)
    P.gaussian_efield(shape, E, 0.7, 22)
    R.init(shape)
    R.set(U, E)
    with tempfile.TemporaryDirectory() as d:
        uf, ef = R.save_configuration(d, "Links", "Fields", 9)
        shutil.copy(uf, os.path.join(HERE, f"ref_config_su{nc}_U.txt"))
        shutil.copy(ef, os.path.join(HERE, f"ref_config_su{nc}_E.txt"))
    np.savez_compressed(os.path.join(HERE, f"ref_config_su{nc}.npz"), U=U, E=E, shape=np.array(shape))


def cooling():
    P, R = oracle.Port(2), oracle.Ref(2)
    shape = (6, 6, 6)
    U, E = oracle.empty_fields(2, shape)
    P.random_links(shape, U, 0.5, 3)
    P.gaussian_efield(shape, E, 0.7, 4)
    P.gauss_restore(shape, U, E, 1e-14, 10000)
    R.init(shape)
    R.set(U, E)
    R.cooling_init(0, 16, 8, np.sqrt(0.02))
    R.cooling_start()
    totals, cooled = [], []
    for _ in range(3):
        R.leapfrog(0.05, 20)
        totals.append(R.cooling_update(1))
        cooled.append(R.cooling_links())
    np.savez_compressed(os.path.join(HERE, "ref_cooling_su2.npz"), U0=U, E0=E, totals=np.array(totals),
                        cooled=np.array(cooled), steps=16, sqrt_dctau=np.sqrt(0.02), dt=0.05, every=20)


def cooling_su3():
    """SU(3) CoolingMethod, the reference's own, its matrix log calling LAPACK's ZGEEV in the
    OpenBLAS that SciPy ships (the restatement in oracle/ref_wrap.cpp where that is absent;
    the fixture records which): cumulative cooled ΔN_CS and cooled links, level 0 at 6^3,
    level 1 at 8^3."""
    lapack = oracle.scipy_lapack()
    if lapack:
        os.environ["TCYM_REF_LAPACK"] = lapack[0]
    P, R = oracle.Port(3), oracle.Ref(3)
    out = {"dt": 0.05, "every": 20, "sqrt_dctau": np.sqrt(0.02),
           "zgeev": lapack[1] if lapack and R.lapack_in_use() else "restated (oracle/ref_wrap.cpp)"}
    for level, shape, steps, bf in ((0, (6, 6, 6), 16, 8), (1, (8, 8, 8), 12, 2)):
        U, E = oracle.empty_fields(3, shape)
        P.random_links(shape, U, 0.4, 7 + level)
        P.gaussian_efield(shape, E, 0.6, 8 + level)
        P.gauss_restore(shape, U, E, 1e-14, 10000)
        R.init(shape)
        R.set(U, E)
        R.cooling_init(level, steps, bf, np.sqrt(0.02))
        R.cooling_start()
        totals, cooled = [], []
        for _ in range(3):
            R.leapfrog(0.05, 20)
            totals.append(R.cooling_update(1))
            cooled.append(R.cooling_links(level))
        out.update({f"U0_{level}": U, f"E0_{level}": E, f"totals{level}": np.array(totals),
                    f"cooled{level}": np.array(cooled), f"steps{level}": steps, f"bf{level}": bf})
    os.environ.pop("TCYM_REF_LAPACK", None)
    np.savez_compressed(os.path.join(HERE, "ref_cooling_su3.npz"), **out)


def cooling_blocked():
    """CoolingMethod with lattice blocking (StandardBlockingLevel 1 and 2) on SU(2) 8^3:
    the cooled ΔN_CS totals and cooled (blocked) links of three updates."""
    P, R = oracle.Port(2), oracle.Ref(2)
    shape = (8, 8, 8)
    U, E = oracle.empty_fields(2, shape)
    P.random_links(shape, U, 0.5, 5)
    P.gaussian_efield(shape, E, 0.7, 6)
    P.gauss_restore(shape, U, E, 1e-14, 10000)
    out = {"U0": U, "E0": E, "dt": 0.05, "every": 20, "sqrt_dctau": np.sqrt(0.02)}
    for level, steps, bf in ((1, 16, 2), (2, 12, 1)):
        R.init(shape)
        R.set(U, E)
        R.cooling_init(level, steps, bf, np.sqrt(0.02))
        R.cooling_start()
        totals, cooled = [], []
        for _ in range(3):
            R.leapfrog(0.05, 20)
            totals.append(R.cooling_update(1))
            cooled.append(R.cooling_links(level))
        out[f"totals{level}"] = np.array(totals)
        out[f"cooled{level}"] = np.array(cooled)
        out[f"steps{level}"] = steps
        out[f"bf{level}"] = bf
    np.savez_compressed(os.path.join(HERE, "ref_cooling_blocked_su2.npz"), **out)


def cooling_su2_96():
    shape = (96, 96, 96)
    R = oracle.Ref(2)
    R.init(shape)
    R.set_zero()
    R.thermal_efield(2.0, 4)  # E = N(0,1)/sqrt(2) (seed 4), then Restore
    R.leapfrog(0.05, 2000)
    U, E = R.get()
    rng = np.random.default_rng(96)
    idx = rng.choice(U.shape[0], size=64, replace=False)
    out = {"start_obs": R.observables(), "fp_sites": idx, "fp_U": U[idx].copy(), "fp_E": E[idx].copy(),
           "dtau": 0.02, "every": 10, "sweeps": 500}
    sim, tot = [], 0.0
    for _ in range(50):
        tot += R.flow(np.sqrt(0.02), 10, 1)
        o = R.observables()
        sim.append([o[0], o[1], o[2], tot])
    out["simultaneous"] = np.array(sim)
    P = oracle.Port(2)
    cb, tot = [], 0.0
    for _ in range(50):
        tot += P.flow_checkerboard_cal(shape, U, E, 0.02, 10, 1)
        o = P.observables(shape, U, E)
        cb.append([o[0], o[1], o[2], tot])
    out["checkerboard"] = np.array(cb)
    np.savez_compressed(os.path.join(HERE, "ref_cooling_su2_96.npz"), **out)


GENERATORS = ("states", "group", "leapfrog_series_su2_16", "thermalize", "cooling", "cooling_blocked", "cooling_su3",
              "configuration", "cooling_su2_96")


if __name__ == "__main__":
    oracle.build()
    if not (oracle.ref_available(2) and oracle.ref_available(3)):
        sys.exit("the reference's sources must be compiled first: make -C oracle ref")
    which = sys.argv[1:] or GENERATORS  # e.g. `make_golden.py cooling_su2_96` regenerates one fixture
    for name in which:
        fn = globals()[name]
        if name in ("states", "group", "thermalize", "configuration"):
            for nc in (2, 3):
                fn(nc)
        else:
            fn()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
