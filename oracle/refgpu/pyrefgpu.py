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
CAGES_CUBIN = os.path.join(REF_DIR, "ref_cages.cubin")
LIB = os.path.join(REF_DIR, "librefgpu.so")
_lib = None


def build_host(quiet=True):
    """Compile the host harness (needs nvcc and a cubin built from the reference)."""
    if not os.path.exists(CUBIN):
        return None
    cmd = [os.environ.get("NVCC", "nvcc"), "-shared", "-Xcompiler", "-fPIC", "-O2", "-std=c++17",
           "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB, os.path.join(HERE, "ref_gpu.cu"),
           os.path.join(HERE, "ref_cages.cu")]
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
        L.refgpu_set_trace.argtypes = [P, P, I]
        L.refgpu_error.restype = ctypes.c_char_p
        L.refgpu_cages_set_cubin.argtypes = [P, ctypes.c_size_t]
        L.refgpu_cages_setup.argtypes = [I, I, I, D, D, D, P]
        L.refgpu_cages_sizes.argtypes = [P]
        L.refgpu_build_cages.argtypes = [I, I, P, P, P, P, P, P, ctypes.POINTER(D)]
        L.refgpu_cages_error.restype = ctypes.c_char_p
        if os.path.exists(CAGES_CUBIN):
            cdata = open(CAGES_CUBIN, "rb").read()
            cbuf = ctypes.create_string_buffer(cdata, len(cdata))
            L._cages_cubin = cbuf
            L.refgpu_cages_set_cubin(cbuf, len(cdata))
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

    def solve(self, rhs, residual, max_iter=20000, trace=0):
        """rhs: the reference's -b (dense); returns (phi, niter, resid, ms, status),
        and with trace > 0 also (alpha, beta) of its first `trace` iterations (NaN
        past the last)."""
        L = lib()
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        phi = np.empty(self.shape, np.float64)
        it, res, ms = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        ta, tb = np.full(max(trace, 1), np.nan), np.full(max(trace, 1), np.nan)
        L.refgpu_set_trace(ta.ctypes.data if trace else None, tb.ctypes.data if trace else None, trace)
        try:
            rc = L.refgpu_solve(rhs.ctypes.data, residual, max_iter, phi.ctypes.data, ctypes.byref(it),
                                ctypes.byref(res), ctypes.byref(ms))
        finally:
            L.refgpu_set_trace(None, None, 0)
        if rc not in (0, 11, 12):
            raise RuntimeError("refgpu_solve %d: %s" % (rc, L.refgpu_error().decode()))
        if trace:
            return phi, it.value, res.value, ms.value, rc, (ta[:trace].copy(), tb[:trace].copy())
        return phi, it.value, res.value, ms.value, rc

    def close(self):
        lib().refgpu_free()


def cages_available():
    return available() and os.path.exists(CAGES_CUBIN)


class RefCages:
    """The reference's cage builder (cuda_build_cages around its own kernels of
    src/particle_kernel.cu) on one GPU for one grid (bc: W,E,S,N,B,T with 0
    periodic / 2 Neumann)."""

    def __init__(self, nx, ny, nz, dx, dy, dz, bc):
        L = lib()
        rc = L.refgpu_cages_setup(nx, ny, nz, dx, dy, dz, (ctypes.c_int * 6)(*bc))
        if rc:
            raise RuntimeError("refgpu_cages_setup %d: %s" % (rc, L.refgpu_cages_error().decode()))
        sz = np.zeros(10, np.int64)
        L.refgpu_cages_sizes(sz.ctypes.data)
        self.sizes = [int(v) for v in sz[:4]]
        self.part_bytes, self.off_n, self.off_r, self.off_x, self.off_y, self.off_z = (int(v) for v in sz[4:10])

    def parts_bytes(self, xyzr):
        """(n, 4) rows x, y, z, r -> the reference's part_struct array as bytes."""
        xyzr = np.asarray(xyzr, np.float64).reshape(-1, 4)
        raw = np.zeros((max(len(xyzr), 1), self.part_bytes), np.uint8)
        for n, (x, y, z, r) in enumerate(xyzr):
            raw[n, self.off_n:self.off_n + 4] = np.frombuffer(np.int32(n).tobytes(), np.uint8)
            for off, v in ((self.off_r, r), (self.off_x, x), (self.off_y, y), (self.off_z, z)):
                raw[n, off:off + 8] = np.frombuffer(np.float64(v).tobytes(), np.uint8)
        return raw

    def build(self, xyzr, with_parts=True):
        """Returns (phase, phase_shell, flag_u, flag_v, flag_w, ms): the
        reference's ghosted arrays (flat) and the device time of the builder."""
        L = lib()
        xyzr = np.asarray(xyzr, np.float64).reshape(-1, 4)
        raw = np.ascontiguousarray(self.parts_bytes(xyzr))
        out = [np.zeros(self.sizes[0], np.int32), np.zeros(self.sizes[0], np.int32),
               np.zeros(self.sizes[1], np.int32), np.zeros(self.sizes[2], np.int32), np.zeros(self.sizes[3], np.int32)]
        ms = ctypes.c_double()
        rc = L.refgpu_build_cages(1 if with_parts else 0, len(xyzr), raw.ctypes.data, *[a.ctypes.data for a in out],
                                  ctypes.byref(ms))
        if rc:
            raise RuntimeError("refgpu_build_cages %d: %s" % (rc, L.refgpu_cages_error().decode()))
        return (*out, ms.value)

    def close(self):
        lib().refgpu_cages_free()
