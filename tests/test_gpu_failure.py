"""Failure detection without a GPU fault: the TMA search kernel's bounded
waits.  bbpp_debug_wait shortens the bound and makes the kernel's first CTA
leave one plane's copies unissued, so its wait for them runs out; the CTA
drains, the solve stops with DONE_TIMEOUT and the host reports
BBPP_WAIT_TIMEOUT.  The context must stay usable: the next solve, with the
hook off, converges.  Nothing faults, traps or hangs."""
import numpy as np
import pytest

import bbpp

pytestmark = pytest.mark.gpu
P, N = bbpp.PERIODIC, bbpp.NEUMANN


def problem(dims, bc, seed):
    nx, ny, nz = dims
    g = bbpp.Grid.make(nx, ny, nz, 1.0 / nx, 1.0 / ny, 1.0 / nz, bc)
    rng = np.random.default_rng(seed)
    mask = (rng.random(g.shape) < 0.05).astype(np.uint8)
    b = rng.uniform(-1, 1, g.shape)
    b[mask == 1] = 0
    b[mask == 0] -= b[mask == 0].mean()
    return g, mask, b


def test_solve_reports_wait_timeout_and_recovers(bbpp_lib):
    g, mask, b = problem((64, 64, 32), (P, P, P, P, N, N), 3)   # a grid the TMA kernel takes
    s = bbpp.Solver(g)
    L = bbpp.lib()
    assert L.bbpp_debug_wait(s.handle, 2_000_000, 1) == 0       # 2 ms bound, hook on
    x, rep = s.solve_host(b, mask, tol=1e-8, precision=bbpp.FP32_IR, ok=(bbpp.WAIT_TIMEOUT,))
    assert rep.status == bbpp.WAIT_TIMEOUT
    assert L.bbpp_debug_wait(s.handle, 0, 0) == 0
    x, rep = s.solve_host(b, mask, tol=1e-8, precision=bbpp.FP32_IR)
    assert rep.status == bbpp.CONVERGED and rep.true_rel <= 1e-8 * 1.01
    # FP64 runs no TMA kernel: the hook leaves it alone
    assert L.bbpp_debug_wait(s.handle, 2_000_000, 1) == 0
    x, rep = s.solve_host(b, mask, tol=1e-10, precision=bbpp.FP64)
    assert rep.status == bbpp.CONVERGED
    L.bbpp_debug_wait(s.handle, 0, 0)


def test_search_step_reports_wait_timeout(bbpp_lib):
    g, mask, b = problem((128, 16, 8), (P,) * 6, 4)
    s = bbpp.Solver(g)
    L = bbpp.lib()
    r = bbpp.DeviceArray.from_host(b.astype(np.float32))
    z = bbpp.DeviceArray(g.shape, np.float32)
    m = bbpp.DeviceArray.from_host(mask)
    L.bbpp_debug_wait(s.handle, 1_000_000, 1)
    with pytest.raises(bbpp.BbppError) as e:
        s.search_step(r, r, z, z, z, m, first=True, precision=bbpp.FP32_IR, kernel=2)
    assert e.value.status == bbpp.WAIT_TIMEOUT
    L.bbpp_debug_wait(s.handle, 0, 0)
    s.search_step(r, r, z, z, z, m, first=True, precision=bbpp.FP32_IR, kernel=2)   # usable again
