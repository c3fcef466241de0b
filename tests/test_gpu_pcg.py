"""GPU parity of the CUDA path against the CPU oracle, through the C ABI.

Kernel level: (-A)p, invM, residual and the sphere mask on odd, tile-edge and
tiny grids, periodic seams and Neumann walls, masks touching both.
Solve level: the FP64 method against the oracle's PCG on the same inputs
(solutions compared to 1e-10 relative after both reach 1e-13), the reference
(r,z) stopping rule, error statuses, and the FP32-inner method.
"""
import numpy as np
import pytest

import bbpp
from bbpp import problems

pytestmark = pytest.mark.gpu
P, N = bbpp.PERIODIC, bbpp.NEUMANN

SHAPES = [
    ((5, 7, 3), (P,) * 6),
    ((17, 40, 9), (P, P, P, P, N, N)),
    ((33, 33, 33), (N,) * 6),
    ((32, 8, 16), (P, P, N, N, P, P)),
    ((64, 24, 12), (N, N, P, P, N, N)),
    ((1, 9, 4), (P,) * 6),
]


def rand_mask(shape, seed, frac=0.15):
    rng = np.random.default_rng(seed)
    return (rng.random(shape) < frac).astype(np.uint8)


def to_orc(orc, g):
    return orc.from_tuple(g.as_tuple())


@pytest.fixture(scope="module")
def lib(bbpp_lib):
    return bbpp_lib


@pytest.mark.parametrize("dims,bc", SHAPES)
@pytest.mark.parametrize("masked", [False, True])
def test_spmv_matches_oracle(lib, orc, dims, bc, masked):
    nx, ny, nz = dims
    g = bbpp.Grid.make(nx, ny, nz, 1.0 / nx, 1.3 / ny, 0.7 / nz, bc)
    s = bbpp.Solver(g)
    rng = np.random.default_rng(nx * 31 + ny)
    p = rng.normal(size=g.shape)
    mask = rand_mask(g.shape, nz) if masked else None
    if masked:
        p[mask == 1] *= 0.5
    dp = bbpp.DeviceArray.from_host(p)
    dA = bbpp.DeviceArray(g.shape, np.float64)
    dm = bbpp.DeviceArray.from_host(mask) if masked else None
    s.spmv(dp, dA, dm)
    got = dA.download()
    ref = orc.spmv(to_orc(orc, g), p, mask)
    scale = np.abs(p).max() * max(g.dx, g.dy, g.dz) ** -2 * 6
    assert np.abs(got - ref).max() <= 1e-14 * scale


@pytest.mark.parametrize("dims,bc", SHAPES)
def test_invm_bit_exact(lib, orc, dims, bc):
    nx, ny, nz = dims
    g = bbpp.Grid.make(nx, ny, nz, 1.0 / nx, 1.0 / ny, 1.0 / nz, bc)
    s = bbpp.Solver(g)
    d = bbpp.DeviceArray(g.shape, np.float64)
    s.invm(d)
    assert np.array_equal(d.download(), orc.invm(to_orc(orc, g)))


@pytest.mark.parametrize("n,bc,nsph,rad", [(32, "ppn", 6, 3.5), (45, "ppp", 9, 4.2), (24, "nnn", 3, 5.0),
                                           (64, "ppn", 40, 4.0)])
def test_sphere_mask_bit_exact(lib, orc, n, bc, nsph, rad):
    g = problems.make_grid(n, bc)
    cents, radii = problems.place_spheres(g, nsph, rad, seed=n)
    # push one sphere across the periodic seam / close to a wall
    cents[0, 0] = 0.3 * g.dx
    s = bbpp.Solver(g)
    dm = bbpp.DeviceArray(g.shape, np.uint8)
    s.sphere_mask(cents, radii, dm)
    got = dm.download()
    ref = orc.sphere_mask(to_orc(orc, g), cents, radii)
    assert np.array_equal(got, ref)
    assert np.array_equal(problems.sphere_mask_host(g, cents, radii), ref)
    assert got.sum() > 0


def test_residual_matches_oracle(lib, orc):
    g = problems.make_grid(40, "ppn")
    mask = rand_mask(g.shape, 5, 0.05)
    rng = np.random.default_rng(7)
    b, x = rng.normal(size=g.shape), rng.normal(size=g.shape)
    s = bbpp.Solver(g)
    db, dx, dr = bbpp.DeviceArray.from_host(b), bbpp.DeviceArray.from_host(x), bbpp.DeviceArray(g.shape, np.float64)
    dm = bbpp.DeviceArray.from_host(mask)
    rr, bb = s.residual(db, dx, dr, dm)
    ref = b - orc.spmv(to_orc(orc, g), x, mask)
    assert np.abs(dr.download() - ref).max() <= 1e-13 * np.abs(ref).max()
    assert abs(rr - (ref * ref).sum()) <= 1e-12 * rr
    assert abs(bb - (b * b).sum()) <= 1e-12 * bb


def _solve_pair(orc, name, n, tol, **kw):
    g, mask, rhs, _ = problems.make_problem(name, n=n)
    s = bbpp.Solver(g)
    x, rep = s.solve_host(rhs, mask, tol=tol, **kw)
    xo, res = orc.pcg(to_orc(orc, g), rhs, mask, tol=tol, stop=kw.get("stop", 1))
    return g, mask, rhs, x, rep, xo, res


@pytest.mark.parametrize("name,n", [("C1", 32), ("C2", 48), ("C4", 40)])
def test_solve_matches_oracle(lib, orc, name, n):
    g, mask, rhs, x, rep, xo, res = _solve_pair(orc, name, n, 1e-13)
    assert rep.status == bbpp.CONVERGED and res["status"] == 0
    assert rep.true_rel <= 1e-13 * 1.01
    if mask is None:  # all-periodic, singular: compare modulo the mean
        x, xo = x - x.mean(), xo - xo.mean()
    else:
        assert np.all(x[mask == 1] == 0)
    err = np.linalg.norm(x - xo) / np.linalg.norm(xo)
    assert err <= 1e-10, err
    assert abs(rep.iters - res["iters"]) <= max(2, res["iters"] // 50)


def test_reference_stop_rule(lib, orc):
    """(r,z) <= pp_residual^2 (rhs,rhs) (src/cuda_solver.cu:235)."""
    g, mask, rhs, x, rep, xo, res = _solve_pair(orc, "C2", 32, 1e-6, stop=bbpp.STOP_REF_RZ)
    assert rep.status == bbpp.CONVERGED
    assert rep.rz <= 1e-12 * rep.bb
    assert abs(rep.iters - res["iters"]) <= 1
    assert np.linalg.norm(x - xo) <= 1e-8 * np.linalg.norm(xo)


def test_status_codes(lib):
    g = problems.make_grid(24, "ppn")
    s = bbpp.Solver(g)
    rhs = problems.uniform_rhs(g.shape, 3)
    x, rep = s.solve_host(rhs, tol=1e-14, max_iter=5, ok=(bbpp.MAX_ITER,))
    assert rep.status == bbpp.MAX_ITER and rep.iters == 6
    x, rep = s.solve_host(np.zeros(g.shape), ok=(bbpp.TINY_RHS,))
    assert rep.status == bbpp.TINY_RHS and rep.iters == 0
    bad = rhs.copy()
    bad[3, 4, 5] = np.nan
    x, rep = s.solve_host(bad, ok=(bbpp.NAN, bbpp.TINY_RHS, bbpp.MAX_ITER))
    assert rep.status in (bbpp.NAN, bbpp.TINY_RHS)
    with pytest.raises(bbpp.BbppError):
        s.solve_host(rhs, tol=-1.0)


def test_warm_start_and_repeat(lib, orc):
    g, mask, rhs, _ = problems.make_problem("C2", n=40)
    s = bbpp.Solver(g)
    x1, r1 = s.solve_host(rhs, mask, tol=1e-10)
    x2, r2 = s.solve_host(rhs, mask, tol=1e-10)
    assert r1.iters == r2.iters and np.array_equal(x1, x2)  # deterministic reductions
    x3, r3 = s.solve_host(rhs, mask, x0=x1, tol=1e-10, guess=bbpp.GUESS_GIVEN)
    assert r3.status == bbpp.CONVERGED and r3.iters <= 1


@pytest.mark.parametrize("ir_mode", [bbpp.IR_RELIABLE, bbpp.IR_RESTART])
@pytest.mark.parametrize("name,n,tol", [("C2", 64, 1e-8), ("C3", 96, 1e-8), ("C1", 32, 1e-10)])
def test_fp32_ir_reaches_tolerance(lib, orc, name, n, tol, ir_mode):
    g, mask, rhs, _ = problems.make_problem(name, n=n)
    s = bbpp.Solver(g)
    x, rep = s.solve_host(rhs, mask, tol=tol, precision=bbpp.FP32_IR, ir_mode=ir_mode)
    assert rep.status == bbpp.CONVERGED and rep.true_rel <= tol * 1.01
    assert rep.outer >= 1  # refinement sweeps, or reliable updates (the confirmation is one)
    xo, res = orc.pcg(to_orc(orc, g), rhs, mask, tol=1e-13)
    # what the reference's method gives at the same tolerance: plain FP64 PCG
    x64, _ = s.solve_host(rhs, mask, tol=tol, precision=bbpp.FP64)
    if mask is None:
        x, xo, x64 = x - x.mean(), xo - xo.mean(), x64 - x64.mean()
    err = np.abs(x - xo).max() / np.abs(xo).max()
    err64 = np.abs(x64 - xo).max() / np.abs(xo).max()
    # FP32 iterations with FP64 reliable updates lose no accuracy against the
    # FP64 method at the same tolerance (a factor 10 for the different
    # iterates; the floor, 100 tol, is far below the condition-number bound)
    assert err < max(10 * err64, 100 * tol), (err, err64)


@pytest.mark.parametrize("name,n,bc", [("C3", 64, None), ("C2", 48, None), ("C1", 32, None), ("C3", 64, "nnn")])
def test_ff_residual_matches_fp64(lib, orc, name, n, bc):
    """Reliable-update residuals in float-float arithmetic against FP64: the
    same PCG iterations within a few, both at the tolerance, and the
    solutions as close as the tolerance allows."""
    g, mask, rhs, _ = problems.make_problem(name, n=n)
    if bc is not None:
        g = problems.make_grid(n, bc)
    s = bbpp.Solver(g)
    out = {}
    for ff in (True, False):
        s.set_ff_resid(ff)
        out[ff] = s.solve_host(rhs, mask, tol=1e-8, precision=bbpp.FP32_IR)
    (xf, rf), (xd, rd) = out[True], out[False]
    for rep in (rf, rd):
        assert rep.status == bbpp.CONVERGED and rep.true_rel <= 1e-8 * 1.01
    assert abs(rf.iters - rd.iters) <= max(3, rd.iters // 50)
    assert rf.outer == rd.outer
    if mask is None:
        xf, xd = xf - xf.mean(), xd - xd.mean()
    assert np.abs(xf - xd).max() <= 1e-5 * np.abs(xd).max()


# grids the TMA kernels take (nx in 32 .. 256, a power of two), where the fused form exists
@pytest.mark.parametrize("name,n,bc", [("C3", 64, None), ("C2", 128, None), ("C1", 32, None), ("C3", 64, "nnn"),
                                       ("C3", 64, "pnp")])
def test_fused_iteration_matches_two_kernels(lib, orc, name, n, bc):
    """The fused FP32 iteration (pending update and search step in one kernel,
    beta from the one-step expansion) against the search + update kernels:
    the same PCG iterations within a few, both at the tolerance, the same
    solution to well within the tolerance's reach."""
    g, mask, rhs, _ = problems.make_problem(name, n=n)
    if bc is not None:
        g = problems.make_grid(n, bc)
    s = bbpp.Solver(g)
    out = {}
    for fused in (True, False):
        s.set_fused(fused)
        out[fused] = s.solve_host(rhs, mask, tol=1e-8, precision=bbpp.FP32_IR)
    (xf, rf), (x2, r2) = out[True], out[False]
    for rep in (rf, r2):
        assert rep.status == bbpp.CONVERGED and rep.true_rel <= 1e-8 * 1.01
    assert abs(rf.iters - r2.iters) <= max(3, r2.iters // 50)
    if mask is None:
        xf, x2 = xf - xf.mean(), x2 - x2.mean()
    assert np.abs(xf - x2).max() <= 1e-5 * np.abs(x2).max()
    # the fused path ran: its kernel appears in the kernel statistics
    s.set_fused(True)
    s.set_profiling(True)
    s.solve_host(rhs, mask, tol=1e-8, precision=bbpp.FP32_IR)
    kinds = {k[0] for k in s.kernel_stats()}
    s.set_profiling(False)
    assert "fused_f32" in kinds


@pytest.mark.parametrize("dims,bc", SHAPES)
@pytest.mark.parametrize("precision,ir_mode", [(bbpp.FP64, 0), (bbpp.FP32_IR, bbpp.IR_RELIABLE),
                                               (bbpp.FP32_IR, bbpp.IR_RESTART)])
def test_solve_odd_shapes(lib, orc, dims, bc, precision, ir_mode):
    """Whole solves on odd, tile-edge and tiny grids with every boundary mix,
    masked, in FP64 and in both mixed-precision forms (the search kernel's
    pair and scalar paths, partial tiles, wall classes)."""
    nx, ny, nz = dims
    g = bbpp.Grid.make(nx, ny, nz, 1.0 / nx, 1.0 / ny, 1.0 / nz, bc)
    mask = rand_mask(g.shape, nx + ny, 0.1)
    rng = np.random.default_rng(nx * ny)
    b = rng.uniform(-1, 1, g.shape)
    b[mask == 1] = 0
    b[mask == 0] -= b[mask == 0].mean()
    s = bbpp.Solver(g)
    tol = 1e-10 if precision == bbpp.FP64 else 1e-8
    x, rep = s.solve_host(b, mask, tol=tol, precision=precision, ir_mode=ir_mode)
    assert rep.status == bbpp.CONVERGED and rep.true_rel <= tol * 1.01
    xo, res = orc.pcg(to_orc(orc, g), b, mask, tol=1e-13)
    assert np.all(x[mask == 1] == 0)
    if not mask.any():
        # no solid cell: periodic/Neumann Poisson is singular and the solution
        # is defined up to a constant, which FP32 round-off may shift
        x, xo = x - x.mean(), xo - xo.mean()
    err = np.abs(x - xo).max() / max(np.abs(xo).max(), 1e-300)
    # against the FP64 method at the same tolerance, as in test_fp32_ir_reaches_tolerance
    x64, _ = s.solve_host(b, mask, tol=tol, precision=bbpp.FP64)
    if not mask.any():
        x64 = x64 - x64.mean()
    err64 = np.abs(x64 - xo).max() / max(np.abs(xo).max(), 1e-300)
    assert err < max(10 * err64, 100 * tol), (err, err64)


@pytest.mark.parametrize("name,n,bc", [("C3", 128, None), ("C1", 64, None), ("C2", 64, "nnn")])
@pytest.mark.parametrize("ws_ns", ["3", "4", "6"])
def test_ws_fused_kernel_matches_fused(lib, name, n, bc, ws_ns, monkeypatch):
    """The warp-specialised fused kernel (producer warp, empty barriers, lower
    z neighbour from a register) against the
    fused kernel, chosen per context when it is created, for ring depths of 3,
    4 and 6 stages.  Per cell both compute the same values; the two launches may
    cut z into different chunks, so the dot products sum their CTA partials in a
    different grouping, and the iterates agree to rounding, not bit for bit."""
    g, mask, rhs, _ = problems.make_problem(name, n=n)
    if bc is not None:
        g = problems.make_grid(n, bc)
    monkeypatch.setenv("BBPP_FUSED_WS", "0")
    s_old = bbpp.Solver(g)
    monkeypatch.setenv("BBPP_FUSED_WS", "1")
    monkeypatch.setenv("BBPP_WS_NS", ws_ns)
    s_ws = bbpp.Solver(g)
    x0, r0 = s_old.solve_host(rhs, mask, tol=1e-8, precision=bbpp.FP32_IR)
    x1, r1 = s_ws.solve_host(rhs, mask, tol=1e-8, precision=bbpp.FP32_IR)
    assert r0.status == r1.status == bbpp.CONVERGED
    assert abs(r0.iters - r1.iters) <= 1 and r1.true_rel <= 1e-8 * 1.01
    if mask is None:
        x0, x1 = x0 - x0.mean(), x1 - x1.mean()
    assert np.abs(x0 - x1).max() <= 1e-5 * np.abs(x0).max()


@pytest.mark.parametrize("xsum", [True, False])
@pytest.mark.parametrize("name,n", [("C1", 32), ("C2", 48)])
def test_alpha_beta_trace_matches_oracle(lib, orc, name, n, xsum):
    """The iteration itself against the oracle's PCG on the same inputs:
    alpha_k and beta_k of the first 50 iterations of the plain FP64 method
    agree to 1e-12 relative, with the six-neighbour sums on the integer pipe
    and with FP64 adds.  (The library iterates on the scaled operator, whose
    alpha and beta are the reference's.)"""
    g, mask, rhs, _ = problems.make_problem(name, n=n)
    s = bbpp.Solver(g)
    s.set_xsum(xsum)
    s.set_trace(50)
    x, rep = s.solve_host(rhs, mask, tol=1e-13)
    a, b = s.trace()
    xo, res = orc.pcg(to_orc(orc, g), rhs, mask, tol=1e-13, trace=50)
    assert rep.iters > 50 and res["iters"] > 50
    assert np.isfinite(a).all() and np.isfinite(b).all()
    ra = np.abs(a - res["alpha"]) / np.abs(res["alpha"])
    rb = np.abs(b - res["beta"]) / np.abs(res["beta"])
    assert ra.max() <= 1e-12 and rb.max() <= 1e-12, (ra.max(), rb.max())
    # a later solve without the trace leaves the recorded values alone
    s.set_trace(0)
    s.solve_host(rhs, mask, tol=1e-8)


@pytest.mark.parametrize("dims,spacing,bc", [
    ((64, 40, 32), (1.0, 1.3, 0.8), (P, P, P, P, N, N)),   # 64-wide rows: TMA kernels for FP32
    ((45, 33, 27), (1.0, 0.7, 1.6), (N, N, P, P, N, N)),   # odd sizes: the z-marching kernels
])
def test_anisotropic_solves_match_oracle(lib, orc, dims, spacing, bc):
    """dx != dy != dz: the iteration kernels' non-isotropic forms (three axis
    weights, no integer neighbour sums) in whole solves.  FP64 to 1e-12
    agrees with the oracle's PCG to 1e-9 relative; the FP32 method with FP64
    reliable updates reaches 1e-9 and stays within 100 x tol of it."""
    nx, ny, nz = dims
    g = bbpp.Grid.make(nx, ny, nz, spacing[0] / nx, spacing[1] / ny, spacing[2] / nz, bc)
    mask = rand_mask(g.shape, 11, 0.08)
    rng = np.random.default_rng(12)
    rhs = rng.normal(size=g.shape)
    rhs[mask == 1] = 0
    s = bbpp.Solver(g)
    xo, res = orc.pcg(to_orc(orc, g), rhs, mask, tol=1e-13)
    assert res["status"] == 0
    x64, r64 = s.solve_host(rhs, mask, tol=1e-12, precision=bbpp.FP64)
    assert r64.status == bbpp.CONVERGED and r64.true_rel <= 1e-12 * 1.01
    assert np.all(x64[mask == 1] == 0)
    assert np.linalg.norm(x64 - xo) <= 1e-9 * np.linalg.norm(xo)
    x32, r32 = s.solve_host(rhs, mask, tol=1e-9, precision=bbpp.FP32_IR)
    assert r32.status == bbpp.CONVERGED and r32.true_rel <= 1e-9 * 1.01
    assert np.abs(x32 - xo).max() <= 100 * 1e-9 * np.abs(xo).max()


@pytest.mark.parametrize("dims", [(1024, 32, 12), (768, 16, 10), (512, 24, 9)])
def test_wide_row_fp32_paths_match_oracle(lib, orc, dims):
    """Rows of 512 and 1024 cells take the TMA kernels on 2-row slabs through
    4-D tensor maps (1024: two float4 per thread and plane); 768 cells take the
    z-marching kernels.  The FP32 method with FP64 reliable updates to 1e-9
    against the oracle's FP64 PCG to 1e-13."""
    nx, ny, nz = dims
    g = bbpp.Grid.make(nx, ny, nz, 1.0 / nx, 1.0 / nx, 1.0 / nx, (P, P, P, P, N, N))
    mask = rand_mask(g.shape, nx, 0.05)
    rng = np.random.default_rng(nz)
    rhs = rng.normal(size=g.shape)
    rhs[mask == 1] = 0
    s = bbpp.Solver(g)
    xo, res = orc.pcg(to_orc(orc, g), rhs, mask, tol=1e-13)
    assert res["status"] == 0
    x, rep = s.solve_host(rhs, mask, tol=1e-9, precision=bbpp.FP32_IR)
    assert rep.status == bbpp.CONVERGED and rep.true_rel <= 1e-9 * 1.01
    assert np.all(x[mask == 1] == 0)
    assert np.abs(x - xo).max() <= 100 * 1e-9 * np.abs(xo).max()
