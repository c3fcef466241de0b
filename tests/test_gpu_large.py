"""The largest configured grid: C5, 512^3 cells (134M), periodic x/y, Neumann
z, 4000 spheres of radius 5 cells.  At nx = 512 the FP32 search kernel takes
its 4-D tensor-map path (x split into 256-wide pieces); both methods must
reach 1e-8 true relative residual and agree to the accuracy that residual
implies.  (A uniform random right-hand side keeps the set-up short.)"""
import numpy as np
import pytest

import bbpp
from bbpp import problems

pytestmark = pytest.mark.gpu


def test_c5_512_both_methods(bbpp_lib):
    c = problems.CONFIGS["C5"]
    g = problems.make_grid(c["n"], c["bc"])
    cents, radii = problems.place_spheres(g, c["nsph"], c["rad"], c["seed"])
    s = bbpp.Solver(g)
    dm = bbpp.DeviceArray(g.shape, np.uint8)
    s.sphere_mask(cents, radii, dm)
    mask = dm.download()
    assert mask.sum() > 0.3 * 4000 * 4 / 3 * np.pi * 5 ** 3  # the spheres are there
    rng = np.random.default_rng(5)
    b = rng.uniform(-1, 1, g.shape)
    b[mask == 1] = 0
    b[mask == 0] -= b[mask == 0].mean()
    db = bbpp.DeviceArray.from_host(b)
    del b
    x64 = bbpp.DeviceArray(g.shape, np.float64)
    r64 = s.solve(db, x64, dm, tol=1e-8, precision=bbpp.FP64)
    x32 = bbpp.DeviceArray(g.shape, np.float64)
    r32 = s.solve(db, x32, dm, tol=1e-8, precision=bbpp.FP32_IR)
    assert r64.status == bbpp.CONVERGED and r64.true_rel <= 1e-8 * 1.01
    assert r32.status == bbpp.CONVERGED and r32.true_rel <= 1e-8 * 1.01
    a, c2 = x64.download(), x32.download()
    assert np.all(c2[mask == 1] == 0)
    assert np.linalg.norm(a - c2) <= 1e-4 * np.linalg.norm(a)
    print("C5 512^3: fp64 %d it %.1f ms, mixed %d it %.1f ms" % (r64.iters, r64.ms, r32.iters, r32.ms))
