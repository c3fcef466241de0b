"""bbpp_residual_noalloc: the residual for callers that cannot allocate device
memory while they run (their device buffers are all sized at start-up, or a
fixed memory budget, or a loop that must not call the allocator).  It keeps
its reduction scratch in a static device array instead of a context.

Checked through the C ABI against the context-based bbpp_residual on two
calls in a row (the scratch keeps the previous call's contents, so the second
call shows that what must start at zero is cleared), with the tolerances of
the other residual tests.  The file name sorts last so a run that stops at
the first failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def noalloc_fn(lib):
    f = lib.bbpp_residual_noalloc
    P = ctypes.c_void_p
    f.argtypes = [P, P, P, P, P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), P]
    f.restype = ctypes.c_int
    return f


def test_noalloc_residual_matches_context_residual(bbpp_lib):
    import bbpp
    from bbpp import problems
    f = noalloc_fn(bbpp_lib)
    g = problems.make_grid(40, "ppn", ny=33, nz=27)
    s = bbpp.Solver(g)
    rng = np.random.default_rng(11)
    for call in range(2):
        mask = (rng.random(g.shape) < 0.07 * (call + 1)).astype(np.uint8)
        b = rng.normal(size=g.shape)
        x = rng.normal(size=g.shape) * (call + 1)
        db, dx, dm = bbpp.DeviceArray.from_host(b), bbpp.DeviceArray.from_host(x), bbpp.DeviceArray.from_host(mask)
        r_ref = bbpp.DeviceArray(g.shape, np.float64)
        r_new = bbpp.DeviceArray(g.shape, np.float64)
        rr_ref, bb_ref = s.residual(db, dx, r_ref, dm)
        rr, bb = ctypes.c_double(-1), ctypes.c_double(-1)
        rc = f(ctypes.byref(g), dm.ptr, db.ptr, dx.ptr, r_new.ptr, ctypes.byref(rr), ctypes.byref(bb), None)
        assert rc == bbpp.CONVERGED
        a, e = r_new.download(), r_ref.download()
        assert np.abs(a - e).max() <= 1e-13 * np.abs(e).max()
        assert abs(rr.value - rr_ref) <= 1e-12 * rr_ref
        assert abs(bb.value - bb_ref) <= 1e-12 * bb_ref
    # the particle-free operator (mask NULL)
    r_new = bbpp.DeviceArray(g.shape, np.float64)
    r_ref = bbpp.DeviceArray(g.shape, np.float64)
    rr_ref, bb_ref = s.residual(db, dx, r_ref, None)
    rc = f(ctypes.byref(g), None, db.ptr, dx.ptr, r_new.ptr, ctypes.byref(rr), ctypes.byref(bb), None)
    assert rc == bbpp.CONVERGED
    assert np.abs(r_new.download() - r_ref.download()).max() <= 1e-13 * np.abs(r_ref.download()).max()
    assert abs(rr.value - rr_ref) <= 1e-12 * rr_ref


@pytest.mark.parametrize("nx,ny,nz", [(512, 512, 16), (4096, 512, 2)])
def test_noalloc_residual_z_chunks(bbpp_lib, nx, ny, nz):
    """Grids whose column tiles times planes exceed the scratch's CTA count:
    the stencil launch then gives each CTA a chunk of several planes (512^2 x 16:
    1024 tiles, 2 planes per CTA) or has exactly as many tiles as the scratch
    holds (4096 x 512: 8192 tiles, both planes in one CTA).  Two calls in a row,
    against the context residual."""
    import bbpp
    from bbpp import problems
    f = noalloc_fn(bbpp_lib)
    g = problems.make_grid(nx, "ppn", ny=ny, nz=nz)
    s = bbpp.Solver(g)
    rng = np.random.default_rng(nx + nz)
    for call in range(2):
        mask = (rng.random(g.shape) < 0.05).astype(np.uint8)
        b = rng.normal(size=g.shape)
        x = rng.normal(size=g.shape) * (call + 1)
        db, dx, dm = bbpp.DeviceArray.from_host(b), bbpp.DeviceArray.from_host(x), bbpp.DeviceArray.from_host(mask)
        r_ref = bbpp.DeviceArray(g.shape, np.float64)
        r_new = bbpp.DeviceArray(g.shape, np.float64)
        rr_ref, bb_ref = s.residual(db, dx, r_ref, dm)
        rr, bb = ctypes.c_double(-1), ctypes.c_double(-1)
        rc = f(ctypes.byref(g), dm.ptr, db.ptr, dx.ptr, r_new.ptr, ctypes.byref(rr), ctypes.byref(bb), None)
        assert rc == bbpp.CONVERGED
        a, e = r_new.download(), r_ref.download()
        assert np.abs(a - e).max() <= 1e-13 * np.abs(e).max()
        assert abs(rr.value - rr_ref) <= 1e-12 * rr_ref
        assert abs(bb.value - bb_ref) <= 1e-12 * bb_ref


def test_noalloc_rejects_oversize_grid(bbpp_lib):
    """A grid needing more CTAs than the scratch holds is refused before any
    device work (the pointers are never touched)."""
    import bbpp
    f = noalloc_fn(bbpp_lib)
    g = bbpp.Grid.make(4096, 4096, 2, bc=(0,) * 6)
    d = bbpp.DeviceArray((8,), np.float64)
    rr, bb = ctypes.c_double(), ctypes.c_double()
    rc = f(ctypes.byref(g), None, d.ptr, d.ptr, d.ptr, ctypes.byref(rr), ctypes.byref(bb), None)
    assert rc == bbpp.BAD_ARG
