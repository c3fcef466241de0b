"""Parity against golden vectors produced by the reference's own solver code.

tests/golden/*.npz were written by tests/golden/make_golden.py, which runs the
unmodified src/cuda_solver.cu and src/solver_kernel.cu through their host
build (oracle/ref).  The CPU tests pin the oracle to them; the GPU tests check
the CUDA path against the same vectors.
"""
import glob
import json
import os

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MANIFEST = json.load(open(os.path.join(HERE, "manifest.json")))


def load(name):
    d = dict(np.load(os.path.join(HERE, name + ".npz")))
    d["dims"] = tuple(int(v) for v in d["dims"])
    d["bc"] = tuple(int(v) for v in d["bc"])
    d["h"] = tuple(float(v) for v in d["h"])
    m = d.get("mask")
    d["mask"] = None if m is None or m.size == 0 else m
    return d


def names(kind):
    return sorted(k for k, v in MANIFEST.items() if v["kind"] == kind)


def test_fixtures_present():
    assert len(glob.glob(os.path.join(HERE, "*.npz"))) == len(MANIFEST) >= 9


# ------------------------------------------------------------ oracle (CPU)
@pytest.mark.parametrize("name", names("spmv"))
def test_oracle_spmv_and_invm_bit_exact(orc, name):
    d = load(name)
    g = orc.grid(*d["dims"], *d["h"], bc=d["bc"])
    assert np.array_equal(orc.spmv(g, d["p"], d["mask"]), d["Ap"])
    assert np.array_equal(orc.invm(g), d["invM"])


def test_oracle_rhs_bit_exact(orc):
    d = load("rhs_ppn")
    g = orc.grid(*d["dims"], *d["h"], bc=d["bc"])
    assert np.array_equal(orc.rhs_div(g, float(d["rho_f"]), float(d["dt"]), d["u"], d["v"], d["w"]), d["rhs"])


@pytest.mark.parametrize("name", names("solve"))
def test_oracle_solve_matches_reference(orc, name):
    """Same iterations and, with the reference's (r,z) rule, the same solution
    to round-off (the thrust reduction order is the only difference)."""
    d = load(name)
    g = orc.grid(*d["dims"], *d["h"], bc=d["bc"])
    x, res = orc.pcg(g, d["rhs"], d["mask"], tol=float(d["pp_residual"]), stop=0)
    assert res["status"] == 0
    assert res["iters"] == int(d["niter"])
    assert abs(np.sqrt(res["rz"] / res["bb"]) - float(d["resid"])) <= 1e-6 * float(d["resid"])
    ref = d["phi"]
    assert np.linalg.norm(x - ref) <= 1e-12 * np.linalg.norm(ref)


# ---------------------------------------------------------- CUDA (GPU)
@pytest.mark.gpu
@pytest.mark.parametrize("name", names("spmv"))
def test_gpu_spmv_matches_reference(bbpp_lib, name):
    import bbpp
    d = load(name)
    g = bbpp.Grid.make(*d["dims"], *d["h"], bc=d["bc"])
    s = bbpp.Solver(g)
    dp = bbpp.DeviceArray.from_host(d["p"])
    dA = bbpp.DeviceArray(g.shape, np.float64)
    dm = None if d["mask"] is None else bbpp.DeviceArray.from_host(d["mask"])
    s.spmv(dp, dA, dm)
    scale = np.abs(d["p"]).max() * 6 * max(d["h"]) ** -2 * 4
    assert np.abs(dA.download() - d["Ap"]).max() <= 1e-14 * scale
    di = bbpp.DeviceArray(g.shape, np.float64)
    s.invm(di)
    assert np.array_equal(di.download(), d["invM"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", names("solve"))
def test_gpu_solve_matches_reference(bbpp_lib, name):
    """The reference's stopping rule and pp_residual: iteration count within
    one of the reference's, solution within 1e-10 relative of its solution."""
    import bbpp
    d = load(name)
    g = bbpp.Grid.make(*d["dims"], *d["h"], bc=d["bc"])
    s = bbpp.Solver(g)
    x, rep = s.solve_host(d["rhs"], d["mask"], tol=float(d["pp_residual"]), stop=bbpp.STOP_REF_RZ)
    assert rep.status == bbpp.CONVERGED
    assert abs(rep.iters - int(d["niter"])) <= 1
    ref = d["phi"]
    assert np.linalg.norm(x - ref) <= 1e-10 * np.linalg.norm(ref)


@pytest.mark.parametrize("name", names("epilogue"))
def test_oracle_epilogue_matches_reference(orc, name):
    """Ghosts of phi, projection and pressure update after the solve: the
    oracle's restatement against the reference's kernels (bit for bit; both
    evaluate the same expressions in the same order without contraction)."""
    d = load(name)
    g = orc.grid(*d["dims"], *d["h"], bc=d["bc"])
    u, v, w, p = orc.epilogue(g, d["mask"], float(d["rho_f"]), float(d["dt"]), d["phi"], d["us"], d["vs"], d["ws"],
                              d["p0"])
    for mine, ref in ((u, d["u"]), (v, d["v"]), (w, d["w"]), (p, d["p"])):
        assert mine.shape == ref.shape
        assert np.array_equal(mine, ref)


# ----------------------------------------------------- cage builder (CPU)
@pytest.mark.parametrize("name", names("cages"))
def test_oracle_build_cages_bit_exact(orc, name):
    """The oracle's cuda_build_cages restatement against the reference's own
    cage kernels run through the host build: phase, phase_shell and the three
    face-flag arrays, element for element."""
    d = load(name)
    g = orc.grid(*d["dims"], *d["h"], bc=d["bc"])
    keep = int(d["with_parts"]) == 0
    out = orc.build_cages(g, d["parts"], with_parts=not keep, phase=d["phase"] if keep else None,
                          phase_shell=d["phase_shell"] if keep else None)
    for a, k in zip(out, ("phase", "phase_shell", "flag_u", "flag_v", "flag_w")):
        assert np.array_equal(a, d[k]), k


def test_cage_fixtures_cover_the_cases():
    """Overlapping particles, ghost copies across periodic boundaries, walls,
    odd extents, a particle-free domain."""
    cases = names("cages")
    assert len(cases) >= 5
    assert any(MANIFEST[c]["nparts"] == 0 for c in cases)
    assert all(MANIFEST[c]["shell_cells"] > 0 for c in cases if MANIFEST[c]["nparts"])
