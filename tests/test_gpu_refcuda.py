"""Parity against the reference's own CUDA solver run on the GPU.

oracle/refgpu runs the reference's unmodified kernels (src/solver_kernel.cu,
compiled to oracle/_ref/ref_solver.cubin from the reference tree) under a
restated one-rank host loop of src/cuda_solver.cu.  These tests check:
  * the reference's GPU solve against the golden fixtures, which came from the
    same code run on the CPU (the two runs of the reference agree);
  * this library's FP64 PCG against the reference's GPU solve on identical
    inputs at larger sizes, under the reference's (r,z) stopping rule: the
    same iteration count (within one) and solutions within 1e-10 relative.
Skipped when the cubin is absent (it is built where the reference tree is).
"""
import os
import sys

import numpy as np
import pytest

import bbpp
from bbpp import problems

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "refgpu"))
import pyrefgpu  # noqa: E402

from test_golden import load, names  # noqa: E402

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not pyrefgpu.available(), reason="reference cubin / harness not built")]


@pytest.mark.parametrize("name", names("solve"))
def test_reference_gpu_matches_reference_host_run(bbpp_lib, name):
    d = load(name)
    nx, ny, nz = d["dims"]
    ref = pyrefgpu.RefSolver(nx, ny, nz, *d["h"], d["bc"], d["mask"])
    phi, it, res, ms, rc = ref.solve(d["rhs"], float(d["pp_residual"]))
    ref.close()
    assert rc == 0
    assert abs(it - int(d["niter"])) <= 1
    assert np.linalg.norm(phi - d["phi"]) <= 1e-10 * np.linalg.norm(d["phi"])


@pytest.mark.parametrize("name,n,tol", [("C1", 32, 1e-10), ("C2", 64, 1e-10), ("C3", 96, 1e-8)])
def test_library_matches_reference_gpu(bbpp_lib, name, n, tol):
    g, mask, rhs, _ = problems.make_problem(name, n=n)
    bc = tuple(int(v) for v in g.bc)
    ref = pyrefgpu.RefSolver(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, bc, mask)
    phi, it, res, ms, rc = ref.solve(rhs, tol)
    ref.close()
    assert rc == 0
    s = bbpp.Solver(g)
    x, rep = s.solve_host(rhs, mask, tol=tol, stop=bbpp.STOP_REF_RZ)
    assert rep.status == bbpp.CONVERGED
    assert abs(rep.iters - it) <= 1, (rep.iters, it)
    if mask is None:  # all-periodic without solids: defined up to a constant
        x, phi = x - x.mean(), phi - phi.mean()
    assert np.linalg.norm(x - phi) <= 1e-10 * np.linalg.norm(phi) if tol <= 1e-10 else \
        np.linalg.norm(x - phi) <= 1e-6 * np.linalg.norm(phi)


def full_size_inputs(name):
    """The stated workloads at their full sizes: C2 = 128^3, 64 spheres of
    radius 8 cells, spectral RHS; C3 = 256^3, 1000 spheres of radius 6 cells,
    step 1 of the OU sequence (the benchmark's right-hand side)."""
    if name == "C2":
        g, mask, rhs, _ = problems.make_problem("C2")
        return g, mask, rhs
    c = problems.CONFIGS["C3"]
    g = problems.make_grid(c["n"], c["bc"])
    cents, radii = problems.place_spheres(g, c["nsph"], c["rad"], c["seed"])
    mask = problems.sphere_mask_host(g, cents, radii)
    seq = problems.OUSequence(g.shape, c["seed"], mask)
    seq.field()
    return g, mask, seq.step()


# pp_residual of the reference's rule (r,z) <= pp_residual^2 (b,b): the oracle
# reaches a true relative residual of 3.1e-12 at C2 with 1e-14 (733
# iterations) and 1.2e-12 at C3 with 2e-15 (848 iterations).  Both stay a
# decade above FP64's attainable residual on these grids (C2 with 1e-16 does not
# converge in 5000 iterations), where the (r,z) test would cross the threshold
# at an iteration set by rounding noise.
FULL_SIZE = [("C2", 1e-14), ("C3", 2e-15)]


@pytest.mark.parametrize("name,pp_residual", FULL_SIZE)
def test_library_matches_reference_gpu_full_size(bbpp_lib, name, pp_residual):
    """The FP64 correctness bar at the stated sizes: this library's plain FP64
    PCG and the reference's own CUDA PCG on identical inputs, both under the
    reference's stopping rule, take the same number of iterations (within one)
    and agree to 1e-10 relative."""
    g, mask, rhs = full_size_inputs(name)
    ref = pyrefgpu.RefSolver(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, tuple(int(v) for v in g.bc), mask)
    phi, it, res, ms, rc = ref.solve(rhs, pp_residual)
    ref.close()
    assert rc == 0, rc
    s = bbpp.Solver(g)
    x, rep = s.solve_host(rhs, mask, tol=pp_residual, stop=bbpp.STOP_REF_RZ)
    assert rep.status == bbpp.CONVERGED, rep.as_dict()
    assert abs(rep.iters - it) <= 1, (rep.iters, it)
    assert rep.true_rel <= 1e-11, rep.true_rel
    err = np.linalg.norm(x - phi) / np.linalg.norm(phi)
    assert err <= 1e-10, err
