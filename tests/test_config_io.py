"""Configuration text files in the reference's format (no GPU needed).

IO::SaveConfiguration / IO::LoadConfiguration (IO/SaveConfiguration.cpp:3-56,
IO/LoadConfiguration.cpp:3-120): tcym_write_configuration reproduces the
reference's own files byte for byte (tests/golden/ref_config_su{2,3}_{U,E}.txt,
written by the reference from the arrays in ref_config_su{2,3}.npz), and
tcym_read_configuration reads them back to exactly those arrays; incomplete,
duplicated or out-of-range files are refused."""
import os

import numpy as np
import pytest

import topologicalcymsolver_gb300 as tcym

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("nc", [2, 3])
def test_write_is_the_reference_format(tmp_path, nc):
    d = np.load(os.path.join(G, f"ref_config_su{nc}.npz"))
    shape = tuple(int(v) for v in d["shape"])
    uf, ef = tmp_path / "U.txt", tmp_path / "E.txt"
    tcym.write_configuration(nc, shape, np.ascontiguousarray(d["U"]), np.ascontiguousarray(d["E"]), uf, ef)
    assert uf.read_bytes() == open(os.path.join(G, f"ref_config_su{nc}_U.txt"), "rb").read()
    assert ef.read_bytes() == open(os.path.join(G, f"ref_config_su{nc}_E.txt"), "rb").read()


@pytest.mark.parametrize("nc", [2, 3])
def test_read_reference_files(nc):
    d = np.load(os.path.join(G, f"ref_config_su{nc}.npz"))
    shape = tuple(int(v) for v in d["shape"])
    U, E = tcym.read_configuration(nc, shape, os.path.join(G, f"ref_config_su{nc}_U.txt"),
                                   os.path.join(G, f"ref_config_su{nc}_E.txt"))
    # 15 significant digits: the files hold the arrays to 1e-15 relative
    assert np.abs(U - d["U"]).max() <= 1e-14 and np.abs(E - d["E"]).max() <= 1e-14 * np.abs(d["E"]).max()


def test_read_any_order_and_refusals(tmp_path):
    lines = open(os.path.join(G, "ref_config_su2_E.txt")).read().splitlines()
    shape = (3, 4, 5)
    shuffled = tmp_path / "E.txt"
    rng = np.random.default_rng(0)
    shuffled.write_text("\n".join(lines[i] for i in rng.permutation(len(lines))) + "\n")
    _, E1 = tcym.read_configuration(2, shape, efile=shuffled)
    _, E0 = tcym.read_configuration(2, shape, efile=os.path.join(G, "ref_config_su2_E.txt"))
    assert np.array_equal(E0, E1)
    bad = {"missing": lines[:-1], "duplicate": lines + lines[:1], "outside": lines[:-1] + ["9 0 0 0 1 2 3"],
           "short": lines[:-1] + [" ".join(lines[-1].split()[:-1])]}
    for name, content in bad.items():
        p = tmp_path / f"{name}.txt"
        p.write_text("\n".join(content) + "\n")
        with pytest.raises(tcym.TcymError):
            tcym.read_configuration(2, shape, efile=p)
