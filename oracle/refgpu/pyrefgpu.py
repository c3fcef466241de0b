"""ctypes binding of the GPU run of the reference's pressure solve
(oracle/refgpu/ref_gpu.cu + oracle/_ref/ref_solver.cubin).  Test and
measurement infrastructure: it times and checks against the reference's own
CUDA kernels; the product never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(os.path.dirname(HERE), "_ref")
CUBIN = os.path.join(REF_DIR, "ref_solver.cubin")
LIB = os.path.join(REF_DIR, "librefgpu.so")
_lib = None


def build_host(quiet=True):
    """Compile the host harness (needs nvcc and a cubin built from the reference)."""
    if not os.path.exists(CUBIN):
        return None
    cmd = [os.environ.get("NVCC", "nvcc"), "-shared", "-Xcompiler", "-fPIC", "-O2", "-std=c++17",
           "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB, os.path.join(HERE, "ref_gpu.cu")]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL if quiet else None)
    return LIB


def available():
    return os.path.exists(CUBIN) and os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB)
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.refgpu_set_cubin.argtypes = [P, ctypes.c_size_t]
        L.refgpu_setup.argtypes = [I, I, I, D, D, D, P, P]
        L.refgpu_solve.argtypes = [P, D, I, P, ctypes.POINTER(I), ctypes.POINTER(D), ctypes.POINTER(D)]
        L.refgpu_error.restype = ctypes.c_char_p
        data = open(CUBIN, "rb").read()
        buf = ctypes.create_string_buffer(data, len(data))
        L._cubin = buf
        L.refgpu_set_cubin(buf, len(data))
        _lib = L
    return _lib


class RefSolver:
    """The reference's CUDA PCG on one GPU for one grid (bc: W,E,S,N,B,T with
    0 periodic / 2 Neumann; mask: (nz,ny,nx) uint8 or None)."""

    def __init__(self, nx, ny, nz, dx, dy, dz, bc, mask=None):
        L = lib()
        b = (ctypes.c_int * 6)(*bc)
        m = None
        if mask is not None:
            self._mask = np.ascontiguousarray(mask, dtype=np.uint8)
            m = self._mask.ctypes.data
        rc = L.refgpu_setup(nx, ny, nz, dx, dy, dz, b, m)
        if rc:
            raise RuntimeError("refgpu_setup %d: %s" % (rc, L.refgpu_error().decode()))
        self.shape = (nz, ny, nx)

    def solve(self, rhs, residual, max_iter=20000):
        """rhs: the reference's -b (dense); returns (phi, niter, resid, ms, status)."""
        L = lib()
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        phi = np.empty(self.shape, np.float64)
        it, res, ms = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        rc = L.refgpu_solve(rhs.ctypes.data, residual, max_iter, phi.ctypes.data, ctypes.byref(it), ctypes.byref(res),
                            ctypes.byref(ms))
        if rc not in (0, 11, 12):
            raise RuntimeError("refgpu_solve %d: %s" % (rc, L.refgpu_error().decode()))
        return phi, it.value, res.value, ms.value, rc

    def close(self):
        lib().refgpu_free()
