"""Learned initial guess: data generation, training and use (thin layer over
the bbpp_net_* C ABI; all compute runs in the library's CUDA kernels).

Training data follow the C4 workload: (rhs, previous pressure, converged
pressure) triples of an Ornstein-Uhlenbeck sequence of spectral right-hand
sides on a fixed sphere geometry, solved by the library's own plain FP64 PCG.
"""
import ctypes
import time

import numpy as np

from . import (FP32_IR, FP64, GUESS_GIVEN, GUESS_LEARNED, GUESS_ZERO, DeviceArray, Solver, _check, lib)
from . import problems

_SIG_DONE = False


def _sig():
    global _SIG_DONE
    if _SIG_DONE:
        return lib()
    L = lib()
    P, I, D, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_float
    sig = {
        "bbpp_net_create": (I, [ctypes.c_ulonglong, ctypes.POINTER(P)]),
        "bbpp_net_destroy": (I, [P]),
        "bbpp_net_num_params": (I, [P]),
        "bbpp_net_get_params": (I, [P, P]),
        "bbpp_net_set_params": (I, [P, P]),
        "bbpp_net_loss_grad": (I, [P, I, I, I, I, D, P, P, P, P, ctypes.POINTER(D), P]),
        "bbpp_net_train": (I, [P, I, I, I, I, D, P, P, P, P, I, I, F, ctypes.c_ulonglong, P]),
        "bbpp_net_infer": (I, [P, I, I, I, D, P, P, P, P]),
        "bbpp_net_save": (I, [P, ctypes.c_char_p]),
        "bbpp_net_load": (I, [P, ctypes.c_char_p]),
        "bbpp_conv3": (I, [I, I, P, I, I, P, P, P, I, I, I, I, I, I, I, I, I, I]),
        "bbpp_conv3_wgrad": (I, [I, I, P, I, I, P, I, P, I, I, I, I, I, I, I]),
        "bbpp_conv3_wflip": (I, [I, I, P, P]),
        "bbpp_conv3_tc_launches": (ctypes.c_longlong, []),
        "bbpp_conv3_tc_config": (I, [I, I]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _SIG_DONE = True
    return L


def _p(a):
    return None if a is None else (a.ptr if isinstance(a, DeviceArray) else a)


class Net:
    """The encoder-decoder of the learned guess (parameters on the GPU)."""

    def __init__(self, seed=1):
        L = _sig()
        h = ctypes.c_void_p()
        _check(L.bbpp_net_create(seed, ctypes.byref(h)))
        self.handle = h.value

    def close(self):
        if self.handle:
            _sig().bbpp_net_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self):
        return _sig().bbpp_net_num_params(self.handle)

    def get_params(self):
        out = np.empty(self.num_params, np.float32)
        _check(_sig().bbpp_net_get_params(self.handle, out.ctypes.data))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(_sig().bbpp_net_set_params(self.handle, p.ctypes.data))

    def loss_grad(self, dims, h2, r, prev, target, mask=None, grads=True):
        """dims = (nx, ny, nz); r (residual of prev), prev, target (p* - prev):
        DeviceArrays of nb stacked FP32 volumes; h2 the squared spacing."""
        nx, ny, nz = dims
        nb = r.nbytes // (4 * nx * ny * nz)
        loss = ctypes.c_double()
        g = np.empty(self.num_params, np.float32) if grads else None
        _check(_sig().bbpp_net_loss_grad(self.handle, nx, ny, nz, nb, h2, _p(r), _p(prev), _p(target), _p(mask),
                                         ctypes.byref(loss), None if g is None else g.ctypes.data))
        return loss.value, g

    def train(self, data, steps, batch=4, lr=2e-3, seed=7):
        nx, ny, nz = data.dims
        hist = np.zeros(max(steps, 1), np.float32)
        _check(_sig().bbpp_net_train(self.handle, nx, ny, nz, data.n, data.h2, data.r.ptr, data.prev.ptr,
                                     data.target.ptr, _p(data.mask), steps, batch, lr, seed, hist.ctypes.data))
        return hist[:steps]

    def infer(self, dims, h2, r, prev, mask, out):
        nx, ny, nz = dims
        _check(_sig().bbpp_net_infer(self.handle, nx, ny, nz, h2, _p(r), _p(prev), _p(mask), _p(out)))

    def save(self, path):
        _check(_sig().bbpp_net_save(self.handle, path.encode()))

    def load(self, path):
        _check(_sig().bbpp_net_load(self.handle, path.encode()))


class OUData:
    """Device-resident training samples (FP32): the residual r_t of the warm
    start p_{t-1} for rhs_t, p_{t-1}, and the correction p_t - p_{t-1}."""

    def __init__(self, dims, h2, mask, r, prev, target, seconds):
        self.dims, self.h2, self.mask, self.r, self.prev, self.target = dims, h2, mask, r, prev, target
        self.n = r.shape[0]
        self.gen_seconds = seconds


def ou_sequence_solves(grid, mask_dev, mask_host, nsteps, seed, tol=1e-10, skip=1):
    """Yield (rhs_t, p_t) of an OU sequence solved by plain FP64 PCG (host arrays)."""
    s = Solver(grid)
    seq = problems.OUSequence(grid.shape, seed, mask_host)
    rhs = seq.field()
    drhs = DeviceArray(grid.shape, np.float64)
    dx = DeviceArray(grid.shape, np.float64)
    for t in range(nsteps + skip):
        drhs.upload(rhs)
        rep = s.solve(drhs, dx, mask_dev, tol=tol, precision=FP64)
        if t >= skip:
            yield rhs, dx.download(), rep
        rhs = seq.step()


def make_ou_dataset(n, nsamples, nsph, rad, seed, tol=1e-10, bc="ppn"):
    """C4-style data at n^3: nsph spheres of rad cells, OU spectral rhs,
    p* from plain FP64 PCG; returns OUData (device arrays) and the geometry."""
    t0 = time.time()
    g = problems.make_grid(n, bc)
    cents, radii = problems.place_spheres(g, nsph, rad, seed)
    s = Solver(g)
    dm = DeviceArray(g.shape, np.uint8)
    s.sphere_mask(cents, radii, dm)
    mh = dm.download()
    res = np.zeros((nsamples,) + g.shape, np.float32)
    prev = np.zeros_like(res)
    tgt = np.zeros_like(res)
    db, dp, dr = (DeviceArray(g.shape, np.float64) for _ in range(3))
    last = None
    k = 0
    for rhs, p, rep in ou_sequence_solves(g, dm, mh, nsamples + 1, seed, tol):
        if last is not None and k < nsamples:
            db.upload(rhs)
            dp.upload(last)
            s.residual(db, dp, dr, dm)
            res[k] = dr.download()
            prev[k] = last
            tgt[k] = p - last
            k += 1
        last = p
    data = OUData(g.shape[::-1], g.dx * g.dy, dm, DeviceArray.from_host(res), DeviceArray.from_host(prev),
                  DeviceArray.from_host(tgt), time.time() - t0)
    return data, g, (cents, radii)


def iterations_with(solver, grid, mask, rhs, prev, net=None, tol=1e-8, precision=FP64):
    """PCG iterations from zero, from prev (warm start) and from the learned guess."""
    drhs = DeviceArray.from_host(rhs)
    dprev = DeviceArray.from_host(prev)
    dx = DeviceArray(grid.shape, np.float64)
    out = {}
    r = solver.solve(drhs, dx, mask, tol=tol, precision=precision, guess=GUESS_ZERO)
    out["zero"] = (r.iters, r.ms)
    dx.upload(prev)
    r = solver.solve(drhs, dx, mask, tol=tol, precision=precision, guess=GUESS_GIVEN)
    out["warm"] = (r.iters, r.ms)
    if net is not None:
        r = solver.solve(drhs, dx, mask, tol=tol, precision=precision, guess=GUESS_LEARNED, net=net.handle,
                         prev=dprev.ptr)
        out["learned"] = (r.iters, r.ms, r.guess_ms)
    return out
