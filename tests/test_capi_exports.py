"""The C-ABI library loads without a GPU and exports every function declared in include/*.h."""
import ctypes
import os
import re

import pytest

from topologicalcymsolver_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(inc, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(tcym_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "tcym_leapfrog" in names and "tcym_observables" in names and len(names) > 25


def test_library_exports_every_declared_symbol():
    lib = build.build_library()
    L = ctypes.CDLL(lib)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_version_without_gpu():
    L = ctypes.CDLL(build.build_library())
    assert L.tcym_version() == 100


def test_context_fails_cleanly_without_gpu():
    """On a host without a CUDA device the library reports an error code instead of aborting."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    L = ctypes.CDLL(build.build_library())
    h = ctypes.c_void_p()
    assert L.tcym_ctx_create(0, ctypes.byref(h)) != 0


def test_python_mirror_binds_the_c_abi():
    """Every function of include/tcym.h has a ctypes signature in the Python mirror
    (the no-alloc restore takes device pointers; its callers bind it themselves)."""
    import topologicalcymsolver_gb300 as tcym

    src = open(os.path.join(ROOT, "topologicalcymsolver_gb300", "__init__.py")).read()
    bound = set(re.findall(r'"(tcym_\w+)":\s*\(', src))
    declared = set(declared_functions())
    assert declared - bound == {"tcym_gauss_restore_noalloc"}, sorted(declared - bound)
    assert not bound - declared, sorted(bound - declared)
    assert callable(tcym.pinned_empty)


def test_host_alloc_fails_cleanly_without_gpu():
    """tcym_host_alloc reports an error code (no abort) where the driver has no device;
    tcym_host_free(NULL) is a no-op."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    L = ctypes.CDLL(build.build_library())
    p = ctypes.c_void_p(1)
    L.tcym_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]
    assert L.tcym_host_alloc(1 << 20, ctypes.byref(p)) != 0
    assert not p.value
    assert L.tcym_host_alloc(0, ctypes.byref(p)) == 0 and not p.value
    L.tcym_host_free.argtypes = [ctypes.c_void_p]
    assert L.tcym_host_free(None) == 0


def test_python_structures_match_the_header(tmp_path):
    """The ctypes/numpy mirrors of the header's structures have its sizes and offsets
    (a C program compiled against include/tcym.h prints them)."""
    import shutil
    import subprocess

    import numpy as np

    import topologicalcymsolver_gb300 as tcym

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    src.write_text(
        "#include <stddef.h>\n#include <stdio.h>\n#include \"tcym.h\"\n"
        "int main(void) { printf(\"%zu %zu %zu %zu %zu %zu\\n\", sizeof(tcym_tick), offsetof(tcym_tick, ms),"
        " offsetof(tcym_tick, gap_ms), offsetof(tcym_tick, link_updates), offsetof(tcym_tick, active),"
        " offsetof(tcym_tick, preparing)); return 0; }\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    size, *offs = (int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                                   check=True).stdout.split())
    dt = tcym.TICK_DTYPE
    assert dt.itemsize == size
    assert [dt.fields[n][1] for n in ("ms", "gap_ms", "link_updates", "active", "preparing")] == offs
    assert dt.fields["active"][0] == np.dtype(np.int32)

