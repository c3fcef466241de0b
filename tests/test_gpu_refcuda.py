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
import ctypes
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


@pytest.mark.parametrize("name,n", [("C1", 32), ("C2", 64)])
def test_alpha_beta_trace_matches_reference_gpu(bbpp_lib, name, n):
    """alpha_k and beta_k of the first 50 iterations of this library's FP64
    PCG against those of the reference's own CUDA PCG (its unmodified kernels
    under the restated one-rank loop) on identical inputs: 1e-12 relative."""
    g, mask, rhs, _ = problems.make_problem(name, n=n)
    bc = tuple(int(v) for v in g.bc)
    ref = pyrefgpu.RefSolver(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, bc, mask)
    phi, it, res, ms, rc, (ra, rb) = ref.solve(rhs, 1e-12, trace=50)
    ref.close()
    assert rc == 0 and it > 50
    s = bbpp.Solver(g)
    s.set_trace(50)
    x, rep = s.solve_host(rhs, mask, tol=1e-12, stop=bbpp.STOP_REF_RZ)
    a, b = s.trace()
    assert rep.status == bbpp.CONVERGED
    da = np.abs(a - ra) / np.abs(ra)
    db = np.abs(b - rb) / np.abs(rb)
    assert da.max() <= 1e-12 and db.max() <= 1e-12, (da.max(), db.max())


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


def with_periodic_copies(cents, radii, box, bc):
    """(x, y, z, r) rows of the particles plus, along periodic axes, the shifted
    copy of every particle within two radii of a boundary: the list a one-rank
    Bluebottle run hands its cage builder."""
    rows = [list(c) + [r] for c, r in zip(cents, radii)]
    out = list(rows)
    for row in rows:
        for a in range(3):
            if bc[2 * a] == 0:
                if row[a] < 2 * row[3]:
                    cp = list(row)
                    cp[a] += box[a]
                    out.append(cp)
                elif row[a] > box[a] - 2 * row[3]:
                    cp = list(row)
                    cp[a] -= box[a]
                    out.append(cp)
    return np.array(out, np.float64)


@pytest.mark.skipif(not pyrefgpu.cages_available(), reason="reference cage cubin not built")
@pytest.mark.parametrize("name", ["C3", "C5"])
def test_dropin_cages_match_reference_gpu(bbpp_lib, name):
    """cuda_build_cages of the drop-in against the reference's own cage builder
    (its kernels of src/particle_kernel.cu under a restated one-rank
    cuda_build_cages, compiled without FMA contraction as the host pin is) on
    the same GPU, at the stated geometries: C3 (256^3, 1000 spheres of radius 6
    cells) and C5 (512^3, 4000 spheres of radius 5 cells), with the periodic
    copies the host program adds.  Phase, phase_shell and the three face-flag
    arrays must agree element for element; the two builders' times are
    printed."""
    import time
    from test_dropin import Host, make_dom
    c = problems.CONFIGS[name]
    g = problems.make_grid(c["n"], c["bc"])
    cents, radii = problems.place_spheres(g, c["nsph"], c["rad"], c["seed"])
    box = (g.nx * g.dx, g.ny * g.dy, g.nz * g.dz)
    bc = tuple(int(v) for v in g.bc)
    parts = with_periodic_copies(cents, radii, box, bc)
    ref = pyrefgpu.RefCages(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, bc)
    ref.build(parts)  # warm-up
    *want, ms_ref = ref.build(parts)
    raw = ref.parts_bytes(parts)
    ref.close()
    assert raw.shape[1] == 3128  # BB_PART_STRUCT_BYTES
    H = Host()
    H.dom = make_dom(g.nx, g.ny, g.nz, (g.dx, g.dy, g.dz))
    H.g("dom", ctypes.c_void_p).value = ctypes.addressof(H.dom)
    bcs = (ctypes.c_int * 6).in_dll(H.stub, "bc")
    for i, b in enumerate(bc):
        bcs[i] = b
    H.g("rank", ctypes.c_int).value = 0
    H.g("nprocs", ctypes.c_int).value = 1
    H.g("NPARTS", ctypes.c_int).value = 1
    H.g("nparts", ctypes.c_int).value = len(parts)
    H.g("_parts", ctypes.c_void_p).value = H.dev(raw)
    for nm, a in zip(("_phase", "_phase_shell", "_flag_u", "_flag_v", "_flag_w"), want):
        H.g(nm, ctypes.c_void_p).value = H.dev(np.full(a.shape, 7, np.int32))
    H.lib.cuda_build_cages()  # warm-up
    bbpp.sync()
    best = None
    for _ in range(3):
        t0 = time.perf_counter()
        H.lib.cuda_build_cages()
        bbpp.sync()
        t = (time.perf_counter() - t0) * 1e3
        best = t if best is None else min(best, t)
    print("%s: %d particles; reference cage builder %.2f ms, drop-in %.3f ms (%.0fx)" % (
        name, len(parts), ms_ref, best, ms_ref / best))
    for nm, a in zip(("_phase", "_phase_shell", "_flag_u", "_flag_v", "_flag_w"), want):
        out = np.empty(a.shape, np.int32)
        bbpp.lib().bbpp_d2h(out.ctypes.data, H.g(nm, ctypes.c_void_p).value, out.nbytes)
        assert np.array_equal(out, a), nm
    assert (want[0] > -1).sum() > 0 and (want[1] == 0).sum() > 0
