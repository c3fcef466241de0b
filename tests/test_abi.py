"""CPU checks of the C ABI: the libraries load (or, for the drop-in library
whose Bluebottle globals come from the host program, link) and export every
function their headers declare."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//.*", "", src)
    names = set()
    for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(\w+)\s*\([^;{]*\)\s*;", src, flags=re.M):
        names.add(m.group(1))
    return sorted(n for n in names if not n.startswith("typedef"))


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return {l.split()[-1] for l in out.splitlines() if l.strip()}


def test_core_symbols(bbpp_lib):
    import bbpp
    names = declared("bbpp.h")
    assert "bbpp_solve" in names and "bbpp_create" in names
    syms = exported(bbpp.LIBPATH)
    missing = [n for n in names if n not in syms]
    assert not missing, missing
    for n in names:
        assert hasattr(bbpp_lib, n)


def test_version_and_rng(bbpp_lib):
    import bbpp
    assert b"sm_103a" in bbpp_lib.bbpp_version()
    a = bbpp.rng_uniform(7, 5)
    b = bbpp.rng_uniform(7, 5)
    assert (a == b).all() and ((a >= 0) & (a < 1)).all()


def test_rng_matches_oracle(bbpp_lib, orc):
    """Ranq1 (src/rng.c:25-51) in the library and in the oracle agree."""
    import ctypes
    import bbpp
    L = orc.lib()

    class R(ctypes.Structure):
        _fields_ = [("v", ctypes.c_ulonglong), ("gphase", ctypes.c_int), ("a", ctypes.c_double),
                    ("b", ctypes.c_double), ("c", ctypes.c_double)]
    g = R()
    L.orc_rng_init(ctypes.byref(g), ctypes.c_ulonglong(12345))
    L.orc_rng_dbl.restype = ctypes.c_double
    L.orc_rng_gauss.restype = ctypes.c_double
    ref = [L.orc_rng_dbl(ctypes.byref(g)) for _ in range(4)]
    assert list(bbpp.rng_uniform(12345, 4)) == ref
    L.orc_rng_init(ctypes.byref(g), ctypes.c_ulonglong(99))
    refg = [L.orc_rng_gauss(ctypes.byref(g)) for _ in range(6)]
    assert list(bbpp.rng_gauss(99, 6)) == refg


def test_geometry_rejects_bad_grid(bbpp_lib):
    import bbpp
    g = bbpp.Grid.make(8, 8, 8, bc=(0, 2, 0, 0, 0, 0))
    with pytest.raises(bbpp.BbppError):
        bbpp.Solver(g)
