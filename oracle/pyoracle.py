"""ctypes access to the CPU oracle (liborc.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the solver library or its bindings.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "_build", "liborc.so")


class OrcGrid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("bc", ctypes.c_int * 6)]


class OrcOpts(ctypes.Structure):
    _fields_ = [("stop", ctypes.c_int), ("tol", ctypes.c_double), ("max_iter", ctypes.c_int),
                ("replace_every", ctypes.c_int), ("nonzero_guess", ctypes.c_int), ("trace_len", ctypes.c_int),
                ("trace_alpha", ctypes.c_void_p), ("trace_beta", ctypes.c_void_p)]


class OrcResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iters", ctypes.c_int), ("bb", ctypes.c_double),
                ("rz", ctypes.c_double), ("rr", ctypes.c_double), ("true_rel", ctypes.c_double)]


_L = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _L
    if _L is None:
        if not os.path.exists(LIBPATH):
            build()
        L = ctypes.CDLL(LIBPATH)
        P = ctypes.c_void_p
        L.orc_spmv.argtypes = [ctypes.POINTER(OrcGrid), P, P, P]
        L.orc_invm.argtypes = [ctypes.POINTER(OrcGrid), P]
        L.orc_pcg.argtypes = [ctypes.POINTER(OrcGrid), P, P, P, ctypes.POINTER(OrcOpts), ctypes.POINTER(OrcResult)]
        L.orc_pcg.restype = ctypes.c_int
        L.orc_true_rel.argtypes = [ctypes.POINTER(OrcGrid), P, P, P]
        L.orc_true_rel.restype = ctypes.c_double
        L.orc_dot.argtypes = [ctypes.c_longlong, P, P]
        L.orc_dot.restype = ctypes.c_double
        L.orc_sphere_mask.argtypes = [ctypes.POINTER(OrcGrid), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int, P, P, P, P, P]
        L.orc_rhs_div.argtypes = [ctypes.POINTER(OrcGrid), ctypes.c_double, ctypes.c_double, P, P, P, P]
        L.orc_rhs_mask_refine.argtypes = [ctypes.POINTER(OrcGrid), P, P]
        L.orc_epilogue.argtypes = [ctypes.POINTER(OrcGrid), P, ctypes.c_double, ctypes.c_double, P, P, P, P, P, P, P,
                                   P, P]
        L.orc_rng_fill_uniform.argtypes = [ctypes.c_ulonglong, ctypes.c_longlong, ctypes.c_double, ctypes.c_double, P]
        L.orc_rng_fill_gauss.argtypes = [ctypes.c_ulonglong, ctypes.c_longlong, P]
        L.orc_build_cages.argtypes = [ctypes.POINTER(OrcGrid), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int, ctypes.c_int, P, P, P, P, P, P, P, P, P]
        L.orc_grid_check.argtypes = [ctypes.POINTER(OrcGrid)]
        L.orc_grid_check.restype = ctypes.c_int
        _L = L
    return _L


def grid(nx, ny, nz, dx=None, dy=None, dz=None, bc=(0,) * 6):
    g = OrcGrid()
    g.nx, g.ny, g.nz = nx, ny, nz
    g.dx = 1.0 / nx if dx is None else dx
    g.dy = 1.0 / ny if dy is None else dy
    g.dz = 1.0 / nz if dz is None else dz
    for i, b in enumerate(bc):
        g.bc[i] = b
    return g


def from_tuple(t):
    nx, ny, nz, dx, dy, dz, bc = t
    return grid(nx, ny, nz, dx, dy, dz, bc)


def _p(a):
    return None if a is None else a.ctypes.data


def _c(a, dt):
    return None if a is None else np.ascontiguousarray(a, dtype=dt)


def spmv(g, p, mask=None):
    p = _c(p, np.float64)
    m = _c(mask, np.uint8)
    out = np.empty_like(p)
    lib().orc_spmv(ctypes.byref(g), _p(m), _p(p), _p(out))
    return out


def invm(g):
    out = np.empty((g.nz, g.ny, g.nx))
    lib().orc_invm(ctypes.byref(g), _p(out))
    return out


def pcg(g, rhs, mask=None, tol=1e-10, stop=1, max_iter=20000, replace_every=50, x0=None, trace=0):
    rhs = _c(rhs, np.float64)
    m = _c(mask, np.uint8)
    x = np.zeros_like(rhs) if x0 is None else _c(x0, np.float64).copy()
    o = OrcOpts()
    o.stop, o.tol, o.max_iter, o.replace_every = stop, tol, max_iter, replace_every
    o.nonzero_guess = 0 if x0 is None else 1
    ta = np.zeros(max(trace, 1))
    tb = np.zeros(max(trace, 1))
    o.trace_len = trace
    o.trace_alpha = ta.ctypes.data
    o.trace_beta = tb.ctypes.data
    r = OrcResult()
    lib().orc_pcg(ctypes.byref(g), _p(m), _p(rhs), _p(x), ctypes.byref(o), ctypes.byref(r))
    res = {f: getattr(r, f) for f, _ in OrcResult._fields_}
    if trace:
        res["alpha"] = ta[:trace].copy()
        res["beta"] = tb[:trace].copy()
    return x, res


def true_rel(g, rhs, x, mask=None):
    return lib().orc_true_rel(ctypes.byref(g), _p(_c(mask, np.uint8)), _p(_c(rhs, np.float64)),
                              _p(_c(x, np.float64)))


def sphere_mask(g, cents, radii, origin=(0.0, 0.0, 0.0)):
    c = np.ascontiguousarray(cents, dtype=np.float64).reshape(-1, 3)
    r = np.ascontiguousarray(radii, dtype=np.float64).reshape(-1)
    cx, cy, cz = [np.ascontiguousarray(c[:, i]) for i in range(3)]
    out = np.zeros((g.nz, g.ny, g.nx), np.uint8)
    lib().orc_sphere_mask(ctypes.byref(g), origin[0], origin[1], origin[2], len(r), _p(cx), _p(cy), _p(cz), _p(r),
                          _p(out))
    return out


def rhs_div(g, rho_f, dt, u, v, w):
    out = np.empty((g.nz, g.ny, g.nx))
    lib().orc_rhs_div(ctypes.byref(g), rho_f, dt, _p(_c(u, np.float64)), _p(_c(v, np.float64)),
                      _p(_c(w, np.float64)), _p(out))
    return out


def rhs_mask_refine(g, mask, rhs):
    out = _c(rhs, np.float64).copy()
    lib().orc_rhs_mask_refine(ctypes.byref(g), _p(_c(mask, np.uint8)), _p(out))
    return out


def epilogue(g, mask, rho_f, dt, phi, us, vs, ws, p0):
    """Post-solve steps (ghosts of phi, projection, pressure update): dense
    cells and faces as orc_rhs_div; returns (u, v, w, p)."""
    u = np.empty_like(_c(us, np.float64))
    v = np.empty_like(_c(vs, np.float64))
    w = np.empty_like(_c(ws, np.float64))
    p = np.empty_like(_c(p0, np.float64))
    m = None if mask is None else _c(mask, np.uint8)
    lib().orc_epilogue(ctypes.byref(g), _p(m), ctypes.c_double(rho_f), ctypes.c_double(dt), _p(_c(phi, np.float64)),
                       _p(_c(us, np.float64)), _p(_c(vs, np.float64)), _p(_c(ws, np.float64)),
                       _p(_c(p0, np.float64)), _p(u), _p(v), _p(w), _p(p))
    return u, v, w, p


def rng_uniform(seed, n, lo=0.0, hi=1.0):
    """n draws of the reference's Ranq1 stream for seed, uniform on [lo, hi)."""
    out = np.empty(int(n), np.float64)
    lib().orc_rng_fill_uniform(seed, int(n), lo, hi, out.ctypes.data)
    return out


def rng_gauss(seed, n):
    """n Gaussian draws (polar method) of the reference's Ranq1 stream for seed."""
    out = np.empty(int(n), np.float64)
    lib().orc_rng_fill_gauss(seed, int(n), out.ctypes.data)
    return out


def build_cages(g, parts, with_parts=True, origin=(0.0, 0.0, 0.0), phase=None, phase_shell=None):
    """cuda_build_cages on one rank: parts (n, 4) rows (x, y, z, r); returns the
    ghosted phase, phase_shell and flag_u, flag_v, flag_w arrays (flat, the
    reference's layouts).  Without particles phase and phase_shell are left as
    given (the reference does not touch them then)."""
    parts = np.ascontiguousarray(np.asarray(parts, np.float64).reshape(-1, 4))
    cols = [np.ascontiguousarray(parts[:, i]) for i in range(4)]
    ncc = (g.nx + 2) * (g.ny + 2) * (g.nz + 2)
    ph = np.full(ncc, -1, np.int32) if phase is None else np.array(phase, np.int32).ravel()
    sh = np.ones(ncc, np.int32) if phase_shell is None else np.array(phase_shell, np.int32).ravel()
    fu = np.zeros((g.nx + 3) * (g.nz + 2) * (g.ny + 2), np.int32)
    fv = np.zeros((g.ny + 3) * (g.nx + 2) * (g.nz + 2), np.int32)
    fw = np.zeros((g.nz + 3) * (g.ny + 2) * (g.nx + 2), np.int32)
    ptrs = [c.ctypes.data if len(parts) else None for c in cols]
    lib().orc_build_cages(ctypes.byref(g), origin[0], origin[1], origin[2], int(bool(with_parts)), len(parts), *ptrs,
                          ph.ctypes.data, sh.ctypes.data, fu.ctypes.data, fv.ctypes.data, fw.ctypes.data)
    return ph, sh, fu, fv, fw
