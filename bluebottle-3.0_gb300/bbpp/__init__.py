"""bbpp -- Python binding of the GB300-native Bluebottle pressure-Poisson solver.

The solver is the C ABI in include/bbpp.h, implemented in CUDA for sm_103a in
``libbbpp.so`` (built in-tree by ``build.py``).  This module is a thin ctypes
layer over that ABI; it never falls back to a CPU implementation.  When the
library is missing or no GPU is present, calls that need the device raise.

The operator and method mirror the reference's pressure solve
(src/cuda_solver.cu:38-300, src/solver_kernel.cu): Jacobi PCG on (-A) phi = rhs,
residual replacement every 50 iterations, solid cells as decoupled rows.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(_HERE, "_lib")
LIBPATH = os.path.join(LIBDIR, "libbbpp.so")
DROPIN_LIBPATH = os.path.join(LIBDIR, "libbbpp_bluebottle.so")

PERIODIC = 0
NEUMANN = 2

CONVERGED, TINY_RHS, MAX_ITER, NAN, BAD_ARG, CUDA_ERROR, NO_DEVICE, WAIT_TIMEOUT = range(8)
FP64, FP32_IR = 0, 1
GUESS_ZERO, GUESS_GIVEN, GUESS_LEARNED = 0, 1, 2
STOP_REF_RZ, STOP_TRUE_REL = 0, 1
IR_RELIABLE, IR_RESTART = 0, 1

STATUS_NAMES = {0: "converged", 1: "tiny rhs", 2: "max iterations", 3: "nan residual", 4: "bad argument",
                5: "cuda error", 6: "no device", 7: "device wait timeout"}


class BbppError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__("bbpp: %s%s" % (STATUS_NAMES.get(status, status), (": " + msg) if msg else ""))


class Grid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("bc", ctypes.c_int * 6)]

    @classmethod
    def make(cls, nx, ny, nz, dx=None, dy=None, dz=None, bc=(PERIODIC,) * 6):
        g = cls()
        g.nx, g.ny, g.nz = nx, ny, nz
        g.dx = 1.0 / nx if dx is None else dx
        g.dy = 1.0 / ny if dy is None else dy
        g.dz = 1.0 / nz if dz is None else dz
        for i, b in enumerate(bc):
            g.bc[i] = b
        return g

    @property
    def shape(self):
        return (self.nz, self.ny, self.nx)

    @property
    def n(self):
        return self.nx * self.ny * self.nz

    def as_tuple(self):
        return (self.nx, self.ny, self.nz, self.dx, self.dy, self.dz, tuple(self.bc))


class Opts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("guess", ctypes.c_int), ("stop", ctypes.c_int),
                ("tol", ctypes.c_double), ("max_iter", ctypes.c_int), ("replace_every", ctypes.c_int),
                ("inner_tol", ctypes.c_double), ("max_outer", ctypes.c_int),
                ("net", ctypes.c_void_p), ("prev", ctypes.c_void_p), ("ir_mode", ctypes.c_int), ("ir_drop", ctypes.c_double),
                ("net_coarsen", ctypes.c_int)]


class Report(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iters", ctypes.c_int), ("outer", ctypes.c_int),
                ("replacements", ctypes.c_int), ("bb", ctypes.c_double), ("rz", ctypes.c_double),
                ("rel_resid", ctypes.c_double), ("true_rel", ctypes.c_double), ("ms", ctypes.c_double),
                ("guess_ms", ctypes.c_double), ("bytes", ctypes.c_double), ("launches", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class KStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_int), ("ms", ctypes.c_double),
                ("bytes", ctypes.c_double)]


_lib = None


def lib():
    """Load libbbpp.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise OSError("libbbpp.so not built (run bluebottle-3.0_gb300/build.py): %s" % LIBPATH)
    L = ctypes.CDLL(LIBPATH)
    P, I, D, S = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_size_t
    sig = {
        "bbpp_create": (I, [ctypes.POINTER(Grid), ctypes.POINTER(P)]),
        "bbpp_destroy": (I, [P]),
        "bbpp_set_stream": (I, [P, P]),
        "bbpp_default_opts": (None, [ctypes.POINTER(Opts)]),
        "bbpp_status_str": (ctypes.c_char_p, [I]),
        "bbpp_last_error": (ctypes.c_char_p, [P]),
        "bbpp_solve": (I, [P, P, P, P, ctypes.POINTER(Opts), ctypes.POINTER(Report)]),
        "bbpp_solve_host": (I, [P, P, P, P, ctypes.POINTER(Opts), ctypes.POINTER(Report)]),
        "bbpp_spmv": (I, [P, P, P, P]),
        "bbpp_invm": (I, [P, P]),
        "bbpp_rhs_div": (I, [P, D, D, P, P, P, P]),
        "bbpp_search_step": (I, [P, I, I, P, P, P, P, P, P, D, D, I, I, ctypes.POINTER(D)]),
        "bbpp_residual": (I, [P, P, P, P, P, ctypes.POINTER(D), ctypes.POINTER(D)]),
        "bbpp_sphere_mask": (I, [P, D, D, D, I, P, P, P, P, P]),
        "bbpp_dev_alloc": (I, [S, ctypes.POINTER(P)]),
        "bbpp_dev_free": (I, [P]),
        "bbpp_h2d": (I, [P, P, S]),
        "bbpp_d2h": (I, [P, P, S]),
        "bbpp_memset": (I, [P, I, S]),
        "bbpp_sync": (I, []),
        "bbpp_flush_l2": (I, []),
        "bbpp_fp64_fma_rate": (I, [ctypes.POINTER(D)]),
        "bbpp_stream_mix_rate": (I, [ctypes.c_longlong, ctypes.POINTER(D)]),
        "bbpp_host_alloc": (I, [S, ctypes.POINTER(P)]),
        "bbpp_host_free": (I, [P]),
        "bbpp_kernel_stats": (I, [P, P, I, ctypes.POINTER(I)]),
        "bbpp_set_profiling": (I, [P, I]),
        "bbpp_set_fused": (I, [P, I]),
        "bbpp_set_ff_resid": (I, [P, I]),
        "bbpp_set_xsum": (I, [P, I]),
        "bbpp_set_trace": (I, [P, I]),
        "bbpp_get_trace": (I, [P, P, P, I]),
        "bbpp_neighbour_sums": (I, [P, P, ctypes.c_longlong]),
        "bbpp_neighbour_sums_host": (I, [P, P, ctypes.c_longlong]),
        "bbpp_plan_z_chunks": (I, [ctypes.c_longlong, I, ctypes.c_longlong, I, ctypes.POINTER(I)]),
        "bbpp_rng_uniform": (None, [ctypes.c_ulonglong, ctypes.c_longlong, D, D, P]),
        "bbpp_rng_gauss": (None, [ctypes.c_ulonglong, ctypes.c_longlong, P]),
        "bbpp_version": (ctypes.c_char_p, []),
        "bbpp_set_device": (I, [I]),
        "bbpp_debug_wait": (I, [P, ctypes.c_longlong, I]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, (DeviceArray, DeviceView)):
        return a.ptr
    assert isinstance(a, np.ndarray) and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def _check(rc, ctx=None, ok=(CONVERGED,)):
    if rc not in ok:
        msg = ""
        try:
            msg = (lib().bbpp_last_error(ctx) or b"").decode()
        except Exception:
            pass
        raise BbppError(rc, msg)
    return rc


class DeviceArray:
    """A device allocation made through the C ABI (no torch involved)."""

    def __init__(self, shape, dtype):
        self.shape = tuple(shape) if not np.isscalar(shape) else (int(shape),)
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        p = ctypes.c_void_p()
        _check(lib().bbpp_dev_alloc(max(self.nbytes, 1), ctypes.byref(p)))
        self.ptr = p.value

    @classmethod
    def from_host(cls, a):
        a = np.ascontiguousarray(a)
        d = cls(a.shape, a.dtype)
        d.upload(a)
        return d

    def upload(self, a):
        a = np.ascontiguousarray(a, dtype=self.dtype)
        assert a.nbytes == self.nbytes
        _check(lib().bbpp_h2d(self.ptr, a.ctypes.data, self.nbytes))

    def download(self):
        out = np.empty(self.shape, self.dtype)
        _check(lib().bbpp_d2h(out.ctypes.data, self.ptr, self.nbytes))
        return out

    def zero(self):
        _check(lib().bbpp_memset(self.ptr, 0, self.nbytes))

    def free(self):
        if self.ptr:
            lib().bbpp_dev_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class DeviceView:
    """Device memory owned elsewhere (a CUDA tensor of another library, say),
    passed to the solver by address.  The owner keeps it alive and ordered:
    work on it must be complete before the solver's call reads it."""

    def __init__(self, ptr, owner=None):
        self.ptr = int(ptr)
        self.owner = owner  # kept alive with the view

    @classmethod
    def of_tensor(cls, t):
        """A contiguous CUDA tensor (torch) by its data pointer."""
        assert t.is_cuda and t.is_contiguous()
        return cls(t.data_ptr(), t)


def default_opts(**kw):
    o = Opts()
    lib().bbpp_default_opts(ctypes.byref(o))
    for k, v in kw.items():
        if k == "net" and v is not None and not isinstance(v, int):
            v = v.handle
        if k == "prev" and isinstance(v, DeviceArray):
            v = v.ptr
        setattr(o, k, v)
    return o


class Solver:
    """One solver context (device workspace for one grid)."""

    def __init__(self, grid):
        self.grid = grid
        h = ctypes.c_void_p()
        _check(lib().bbpp_create(ctypes.byref(grid), ctypes.byref(h)))
        self.handle = h.value

    def close(self):
        if self.handle:
            lib().bbpp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, rhs, x, mask=None, ok=(CONVERGED,), **kw):
        """Device-pointer solve; rhs/x/mask are DeviceArrays."""
        o = default_opts(**kw)
        rep = Report()
        rc = lib().bbpp_solve(self.handle, _ptr(mask), _ptr(rhs), _ptr(x), ctypes.byref(o), ctypes.byref(rep))
        _check(rc, self.handle, ok)
        return rep

    def solve_host(self, rhs, mask=None, x0=None, ok=(CONVERGED,), **kw):
        """Host-array solve (copies inside the call); returns (x, report)."""
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        x = np.zeros_like(rhs) if x0 is None else np.ascontiguousarray(x0, dtype=np.float64).copy()
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        o = default_opts(**kw)
        rep = Report()
        rc = lib().bbpp_solve_host(self.handle, _ptr(m), _ptr(rhs), _ptr(x), ctypes.byref(o), ctypes.byref(rep))
        _check(rc, self.handle, ok)
        return x, rep

    def spmv(self, p, Ap, mask=None):
        _check(lib().bbpp_spmv(self.handle, _ptr(mask), _ptr(p), _ptr(Ap)), self.handle)

    def search_step(self, r, pold, pnew, Ap, x, mask=None, beta=0.0, alpha=0.0, first=False, lag=False,
                    precision=FP64, kernel=0):
        """One search-kernel launch (kernel 0 = the solver's choice, 1 = z-marching tiles,
        2 = TMA-staged, FP32 only); returns (p_new, Ap)."""
        pAp = ctypes.c_double()
        _check(lib().bbpp_search_step(self.handle, precision, kernel, _ptr(mask), _ptr(r), _ptr(pold), _ptr(pnew),
                                      _ptr(Ap), _ptr(x), beta, alpha, int(first), int(lag), ctypes.byref(pAp)),
               self.handle)
        return pAp.value

    def rhs_div(self, rho_f, dt, u, v, w, out):
        """rhs = -(rho_f/dt) div u* from dense face DeviceArrays (the reference's PP_rhs)."""
        _check(lib().bbpp_rhs_div(self.handle, rho_f, dt, _ptr(u), _ptr(v), _ptr(w), _ptr(out)), self.handle)

    def invm(self, out):
        _check(lib().bbpp_invm(self.handle, _ptr(out)), self.handle)

    def residual(self, rhs, x, r, mask=None):
        rr, bb = ctypes.c_double(), ctypes.c_double()
        _check(lib().bbpp_residual(self.handle, _ptr(mask), _ptr(rhs), _ptr(x), _ptr(r), ctypes.byref(rr),
                                   ctypes.byref(bb)), self.handle)
        return rr.value, bb.value

    def sphere_mask(self, centres, radii, out, origin=(0.0, 0.0, 0.0)):
        c = np.ascontiguousarray(centres, dtype=np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(radii, dtype=np.float64).reshape(-1)
        cx, cy, cz = [np.ascontiguousarray(c[:, i]) for i in range(3)]
        _check(lib().bbpp_sphere_mask(self.handle, origin[0], origin[1], origin[2], len(r), _ptr(cx), _ptr(cy),
                                      _ptr(cz), _ptr(r), _ptr(out)), self.handle)

    def set_profiling(self, on):
        _check(lib().bbpp_set_profiling(self.handle, 1 if on else 0))

    def set_fused(self, on):
        """FP32 reliable-update iterations as one fused kernel (True) or two."""
        _check(lib().bbpp_set_fused(self.handle, 1 if on else 0))

    def set_ff_resid(self, on):
        """Reliable-update residuals in float-float (True) or FP64 arithmetic."""
        _check(lib().bbpp_set_ff_resid(self.handle, 1 if on else 0))

    def set_xsum(self, on):
        """FP64 stencils on an isotropic grid (the plain iteration's search
        kernel, the FP64 residuals): interior neighbour sums as exact
        fixed-point sums on the integer pipe (True) or FP64 adds."""
        _check(lib().bbpp_set_xsum(self.handle, 1 if on else 0))

    def set_trace(self, n):
        """Record alpha_k, beta_k of the first n iterations of later plain FP64 solves."""
        _check(lib().bbpp_set_trace(self.handle, int(n)))
        self._trace_n = int(n)

    def trace(self):
        """(alpha, beta) of the last plain FP64 solve (NaN past its end)."""
        n = getattr(self, "_trace_n", 0)
        a, b = np.empty(n), np.empty(n)
        _check(lib().bbpp_get_trace(self.handle, a.ctypes.data, b.ctypes.data, n))
        return a, b

    def kernel_stats(self):
        arr = (KStat * 32)()
        n = ctypes.c_int()
        _check(lib().bbpp_kernel_stats(self.handle, ctypes.cast(arr, ctypes.c_void_p), 32, ctypes.byref(n)))
        return [(arr[i].name.decode(), arr[i].launches, arr[i].ms, arr[i].bytes) for i in range(min(n.value, 32))]


class PinnedArray:
    """Page-locked host buffer viewed as a numpy array."""

    def __init__(self, shape, dtype):
        self.dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * self.dtype.itemsize
        p = ctypes.c_void_p()
        _check(lib().bbpp_host_alloc(max(n, 1), ctypes.byref(p)))
        self.ptr = p.value
        buf = (ctypes.c_char * max(n, 1)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            lib().bbpp_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def rng_uniform(seed, n, lo=0.0, hi=1.0):
    out = np.empty(int(n), np.float64)
    lib().bbpp_rng_uniform(seed, int(n), lo, hi, out.ctypes.data)
    return out


def rng_gauss(seed, n):
    out = np.empty(int(n), np.float64)
    lib().bbpp_rng_gauss(seed, int(n), out.ctypes.data)
    return out


def flush_l2():
    _check(lib().bbpp_flush_l2())


def stream_mix_rate(cells):
    """Bytes/s of a streaming kernel with the fused iteration's per-cell traffic
    (bbpp_stream_mix_rate)."""
    v = ctypes.c_double()
    _check(lib().bbpp_stream_mix_rate(int(cells), ctypes.byref(v)))
    return v.value


def plan_z_chunks(units, nz, slots, min_kz):
    """(z-chunks, planes per chunk) the stencil kernels launch with
    (bbpp_plan_z_chunks; host arithmetic, no GPU needed)."""
    kz = ctypes.c_int()
    n = lib().bbpp_plan_z_chunks(int(units), int(nz), int(slots), int(min_kz), ctypes.byref(kz))
    if n < 1:
        raise BbppError(BAD_ARG, "plan_z_chunks")
    return n, kz.value


def neighbour_sums(v, host=False):
    """The FP64 search kernel's neighbour sum of each row of an (n, 6) float64
    array, computed on the GPU (bbpp_neighbour_sums), or by the same code
    compiled for the host (host=True, bbpp_neighbour_sums_host)."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    assert v.ndim == 2 and v.shape[1] == 6
    out = np.empty(v.shape[0], np.float64)
    fn = lib().bbpp_neighbour_sums_host if host else lib().bbpp_neighbour_sums
    _check(fn(v.ctypes.data, out.ctypes.data, v.shape[0]))
    return out


def fp64_fma_rate():
    """FP64 FMAs per second of the current GPU (bbpp_fp64_fma_rate)."""
    v = ctypes.c_double()
    _check(lib().bbpp_fp64_fma_rate(ctypes.byref(v)))
    return v.value


def sync():
    _check(lib().bbpp_sync())
