"""Kernel-level checks of the PCG search kernel (p_new = z + beta p_old,
Ap = L p_new with L = S(-A), (p, Ap), and the lagged x += alpha p_old).

The TMA-staged FP32 kernel and the z-marching tile kernel compute the same
FP32 arithmetic, so their p_new, Ap and x must agree bit for bit; both are
checked against the FP64 oracle's operator (oracle/bbpp_oracle.c, which
restates src/solver_kernel.cu:684-707) on grids with every boundary mix,
partial slabs and the 4-D tensor-map path (nx > 256).
"""
import numpy as np
import pytest

import bbpp

pytestmark = pytest.mark.gpu

P, N = bbpp.PERIODIC, bbpp.NEUMANN

# shapes the TMA kernel takes: nx in {32, 64, 128, 256, 512}, ny a multiple of
# the slab height (1024 / nx rows for nx <= 256, else 4)
TMA_SHAPES = [
    ((32, 32, 8), (P,) * 6),
    ((64, 32, 6), (P, P, N, N, P, P)),
    ((128, 16, 5), (N,) * 6),
    ((256, 12, 4), (P, P, P, P, N, N)),
    ((256, 8, 1), (N, N, P, P, P, P)),
    ((512, 8, 3), (P, P, P, P, N, N)),
    ((32, 64, 3), (N, N, N, N, P, P)),
]


def make(dims, bc, seed):
    nx, ny, nz = dims
    g = bbpp.Grid.make(nx, ny, nz, 1.0 / nx, 1.5 / ny, 0.75 / nz, bc)
    rng = np.random.default_rng(seed)
    mask = (rng.random(g.shape) < 0.1).astype(np.uint8)
    r = rng.uniform(-1, 1, g.shape).astype(np.float32)
    po = rng.uniform(-1, 1, g.shape).astype(np.float32)
    x = rng.uniform(-1, 1, g.shape).astype(np.float32)
    r[mask == 1] = 0
    po[mask == 1] = 0
    return g, mask, r, po, x


def run(s, g, mask, r, po, x, kernel, beta, alpha, first, lag):
    dm = bbpp.DeviceArray.from_host(mask)
    dr, dp, dx = (bbpp.DeviceArray.from_host(a) for a in (r, po, x))
    dpn = bbpp.DeviceArray(g.shape, np.float32)
    dap = bbpp.DeviceArray(g.shape, np.float32)
    pAp = s.search_step(dr, dp, dpn, dap, dx, dm, beta=beta, alpha=alpha, first=first, lag=lag,
                        precision=bbpp.FP32_IR, kernel=kernel)
    return dpn.download(), dap.download(), dx.download(), pAp


@pytest.mark.parametrize("first", [False, True])
@pytest.mark.parametrize("dims,bc", TMA_SHAPES)
def test_tma_search_matches_marched_and_oracle(bbpp_lib, orc, dims, bc, first):
    g, mask, r, po, x = make(dims, bc, sum(dims) + int(first))
    s = bbpp.Solver(g)
    beta, alpha = 0.731, -0.412
    lag = not first
    a = run(s, g, mask, r, po, x, 1, beta, alpha, first, lag)
    b = run(s, g, mask, r, po, x, 2, beta, alpha, first, lag)
    for u, v in zip(a[:3], b[:3]):
        assert np.array_equal(u.view(np.uint32), v.view(np.uint32))
    assert abs(a[3] - b[3]) <= 1e-5 * abs(a[3])
    # against the FP64 operator of the oracle
    pn, Ap, xn, pAp = b
    og = orc.from_tuple(g.as_tuple())
    S = 1.0 / (2 / g.dx ** 2 + 2 / g.dy ** 2 + 2 / g.dz ** 2)
    invm = orc.invm(og)
    z = r.astype(np.float64) * invm / S
    pref = z if first else z + beta * po.astype(np.float64)
    assert np.abs(pn - pref).max() <= 1e-5 * np.abs(pref).max()
    Aref = S * orc.spmv(og, pn.astype(np.float64), mask)
    Aref[mask == 1] = 0
    assert np.all(Ap[mask == 1] == 0)
    assert np.abs(Ap - Aref).max() <= 1e-5 * np.abs(Aref).max()
    xref = x.astype(np.float64) + (alpha * po.astype(np.float64) if lag else 0.0)
    assert np.abs(xn - xref).max() <= 1e-6 * np.abs(xref).max()
    assert abs(pAp - float(np.dot(pn.ravel().astype(np.float64), Ap.ravel()))) <= 1e-5 * abs(pAp)


def test_tma_refuses_other_shapes(bbpp_lib):
    g = bbpp.Grid.make(48, 8, 4, 1 / 48, 1 / 8, 1 / 4, (P,) * 6)
    s = bbpp.Solver(g)
    z = bbpp.DeviceArray(g.shape, np.float32)
    with pytest.raises(bbpp.BbppError):
        s.search_step(z, z, z, z, z, None, first=True, precision=bbpp.FP32_IR, kernel=2)


@pytest.mark.parametrize("dims,bc", TMA_SHAPES[:4])
def test_fp64_search_matches_oracle(bbpp_lib, orc, dims, bc):
    g, mask, r, po, x = make(dims, bc, 7 + sum(dims))
    r, po, x = (a.astype(np.float64) for a in (r, po, x))
    s = bbpp.Solver(g)
    dm = bbpp.DeviceArray.from_host(mask)
    dr, dp, dx = (bbpp.DeviceArray.from_host(a) for a in (r, po, x))
    dpn = bbpp.DeviceArray(g.shape, np.float64)
    dap = bbpp.DeviceArray(g.shape, np.float64)
    beta, alpha = 0.25, 1.5
    pAp = s.search_step(dr, dp, dpn, dap, dx, dm, beta=beta, alpha=alpha, lag=True, precision=bbpp.FP64)
    og = orc.from_tuple(g.as_tuple())
    S = 1.0 / (2 / g.dx ** 2 + 2 / g.dy ** 2 + 2 / g.dz ** 2)
    pref = r * orc.invm(og) / S + beta * po
    pn = dpn.download()
    assert np.abs(pn - pref).max() <= 1e-14 * np.abs(pref).max()
    Aref = S * orc.spmv(og, pn, mask)
    Aref[mask == 1] = 0
    assert np.abs(dap.download() - Aref).max() <= 1e-13 * np.abs(Aref).max()
    assert np.abs(dx.download() - (x + alpha * po)).max() <= 1e-15 * np.abs(x + alpha * po).max()
    assert abs(pAp - float(np.dot(pn.ravel(), dap.download().ravel()))) <= 1e-12 * abs(pAp)


def test_contexts_of_different_grids(bbpp_lib):
    """A context made later for another grid (a smaller TMA stage) leaves an
    earlier context's FP32 solves working."""
    ga = bbpp.Grid.make(128, 16, 16, 1 / 128, 1 / 16, 1 / 16, (P, P, P, P, N, N))
    sa = bbpp.Solver(ga)
    gb = bbpp.Grid.make(32, 32, 8, 1 / 32, 1 / 32, 1 / 8, (P,) * 6)
    sb = bbpp.Solver(gb)
    rng = np.random.default_rng(5)
    mask = (rng.random(ga.shape) < 0.05).astype(np.uint8)
    b = rng.uniform(-1, 1, ga.shape)
    b[mask == 1] = 0
    b[mask == 0] -= b[mask == 0].mean()
    x, rep = sa.solve_host(b, mask, tol=1e-8, precision=bbpp.FP32_IR)
    assert rep.status == bbpp.CONVERGED and rep.true_rel <= 1e-8 * 1.01
    mb = np.zeros(gb.shape, np.uint8)
    mb[0, 0, 0] = 1
    bb = rng.uniform(-1, 1, gb.shape)
    bb[mb == 1] = 0
    xb, repb = sb.solve_host(bb, mb, tol=1e-8, precision=bbpp.FP32_IR)
    assert repb.status == bbpp.CONVERGED
