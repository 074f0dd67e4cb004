"""The reference-named C++ layer (include/tcym_compat.hpp) end to end.

tests/compat/driver.cpp is written against the reference's API (Lattice::Init,
InitialConditions::SetZero, ThermalDynamics::ReassignElectricFields,
Dynamics::Update, Observables::Bulk, LangevinDynamics::Update, Cooling::CoolNSave (also with a Block),
GradientFlow::CalibrationUpdate, the E.B operators).  It is compiled with g++
against libtcym.so for SU(2) and SU(3), run on the GPU, and every number it
prints is compared with the FP64 oracle running the same sequence.
"""
import os
import subprocess

import numpy as np
import pytest

import oracle
from topologicalcymsolver_gb300 import build

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
L = 6
TOL = 1e-9


def run_driver(nc, tmp_path):
    lib = build.build_library()
    exe = str(tmp_path / f"driver{nc}")
    subprocess.run(["g++", "-std=c++17", "-O2", f"-DTCYM_NC={nc}", os.path.join(ROOT, "tests", "compat", "driver.cpp"),
                    "-I" + os.path.join(ROOT, "include"), "-L" + os.path.dirname(lib), "-ltcym",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], check=True)
    out = subprocess.run([exe, str(L)], check=True, capture_output=True, text=True).stdout
    rows = {}
    for line in out.splitlines():
        k, *v = line.split()
        rows.setdefault(k, []).append([float(x) for x in v])
    return rows


def close(a, b, tol=TOL):
    return abs(a - b) <= tol * max(1.0, abs(b))


@pytest.mark.parametrize("nc", [2, 3])
def test_reference_style_driver_matches_oracle(oracle_port, nc, tmp_path):
    got = run_driver(nc, tmp_path)
    P = oracle_port[nc]
    shape = (L, L, L)
    site = lambda x, y, z: x + L * (y + L * z)  # noqa: E731
    U, E = oracle.empty_fields(nc, shape)
    P.set_zero(shape, U, E)
    P.gaussian_efield(shape, E, 1.0 / np.sqrt(2.0), 1)
    P.gauss_restore(shape, U, E, 1e-14, 10000)
    for rec, row in enumerate(got["bulk"]):
        if rec:
            P.leapfrog(shape, U, E, 0.05, 10)
        o = P.observables(shape, U, E)
        assert int(row[0]) == 10 * rec
        assert close(row[1], o[0]) and close(row[2], o[1]) and close(row[3], o[2]), (rec, row, o[:3])
    assert close(got["link"][0][0], U[site(1, 2, 3), 1, 0])
    assert close(got["field"][0][0], E[site(2, 1, 0), 2, 1])
    assert close(got["edotb"][0][0], P.edotb_clover(shape, U, E))
    assert close(got["edotb"][0][1], P.edotb_improved(shape, U, E))
    assert abs(got["unitarity"][0][0] - P.observables(shape, U, E)[11]) < 1e-12
    T = 1.0 / (1.0 / 0.6)
    P.langevin(shape, U, E, 0.02, 1.0, T, 3, 0, 5)
    assert close(got["langevin"][0][0], P.observables(shape, U, E)[0])
    dtau = 0.1414213562373095 ** 2
    Uc, Ec = U.copy(), np.zeros_like(E)
    P.flow(shape, Uc, Ec, dtau, 5, 0)
    assert close(got["cooled"][0][0], Uc[0, 0, 0])
    dn = P.flow(shape, U, E, dtau, 3, 1)
    assert close(got["calibration"][0][0], dn) and close(got["calibration"][0][1], 3 * dtau)
    # Cooling::CoolNSave with one Block, then CoolingMethod at StandardBlockingLevel 1
    s = 0.1414213562373095
    half = L // 2
    sb = lambda x, y, z: x + half * (y + half * z)  # noqa: E731
    Ub = P.cool_blocked(shape, U, s, 6, 1, 2)
    assert close(got["cooled_blocked"][0][0], Ub[sb(0, 0, 0), 0, 0])
    assert close(got["cooled_blocked"][0][1], Ub[sb(1, 2, 2), 2, 0])
    old = Ub
    P.leapfrog(shape, U, E, 0.05, 10)
    new = P.cool_blocked(shape, U, s, 6, 1, 2)
    d = P.cooled_delta_ncs((half, half, half), old, new, 1)
    assert abs(got["cooled_ncs"][0][0] - d) <= TOL * max(abs(d), 1e-3), (got["cooled_ncs"], d)
