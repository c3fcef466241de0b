"""Generate the golden fixtures from the reference's own solver code.

Runs the unmodified reference sources (src/cuda_solver.cu, src/solver_kernel.cu)
through their host build in oracle/_ref/libref.so (see oracle/ref/build_ref.py)
on small seeded inputs, and stores inputs and outputs here as .npz:

  spmv_*.npz   p, mask, (-A)p from PP_spmv_shared_load[_noparts]
  invm_*.npz   invM from PP_jacobi_init
  rhs_*.npz    u*, v*, w*, rho_f, dt and the rhs from PP_rhs
  solve_*.npz  rhs, mask, pp_residual, the solution phi and the iteration
               count of cuda_PP_cg / cuda_PP_cg_noparts (stop rule
               (r,z) <= pp_residual^2 (rhs,rhs), residual replacement every 50)

Needs the reference tree; run:  python tests/golden/make_golden.py
"""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "libref.so")
P, N = 0, 2


def load():
    if not os.path.exists(LIB):
        subprocess.run([sys.executable, os.path.join(ROOT, "oracle", "ref", "build_ref.py")], check=True)
    L = ctypes.CDLL(LIB)
    v = ctypes.c_void_p
    L.ref_setup.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 3 + [v, v]
    L.ref_solve.argtypes = [v, ctypes.c_double, ctypes.c_int, v, v, v]
    L.ref_spmv.argtypes = [v, v]
    L.ref_invm.argtypes = [v]
    L.ref_rhs.argtypes = [ctypes.c_double, ctypes.c_double, v, v, v, v]
    L.ref_solve_u.argtypes = [ctypes.c_double, ctypes.c_double, v, v, v, ctypes.c_double, ctypes.c_int, v, v, v]
    L.ref_epilogue.argtypes = [ctypes.c_double] * 3 + [v] * 10
    L.ref_sizes.argtypes = [v]
    return L


def setup(L, dims, h, bc, mask):
    nx, ny, nz = dims
    b = (ctypes.c_int * 6)(*bc)
    L.ref_setup(nx, ny, nz, h[0], h[1], h[2], b, None if mask is None else mask.ctypes.data)


def spheres_mask(dims, h, bc, cents, rads):
    nx, ny, nz = dims
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    X, Y, Z = (x + 0.5) * h[0], (y + 0.5) * h[1], (z + 0.5) * h[2]
    L = np.array([nx * h[0], ny * h[1], nz * h[2]])
    m = np.zeros((nz, ny, nx), np.uint8)
    for (cx, cy, cz), r in zip(cents, rads):
        d = [X - cx, Y - cy, Z - cz]
        for a, per in enumerate((bc[0] == P, bc[2] == P, bc[4] == P)):
            if per:
                d[a] = d[a] - L[a] * np.round(d[a] / L[a])
        m |= (np.sqrt(d[0] ** 2 + d[1] ** 2 + d[2] ** 2) < r).astype(np.uint8)
    return m


def main():
    L = load()
    rng = np.random.default_rng(20261203)
    manifest = {}

    spmv_cases = [
        ("spmv_ppp_nomask", (5, 4, 3), (1 / 5, 1 / 4, 1 / 3), (P,) * 6, False),
        ("spmv_ppn_mask", (9, 7, 6), (1 / 9, 1.3 / 7, 0.7 / 6), (P, P, P, P, N, N), True),
        ("spmv_nnn_mask", (18, 17, 5), (1 / 18, 1 / 17, 1 / 5), (N,) * 6, True),
        ("spmv_pnp_mask", (20, 6, 33), (1 / 20, 1 / 6, 1 / 33), (P, P, N, N, P, P), True),
    ]
    for name, dims, h, bc, masked in spmv_cases:
        nx, ny, nz = dims
        mask = (rng.random((nz, ny, nx)) < 0.2).astype(np.uint8) if masked else None
        setup(L, dims, h, bc, mask)
        p = rng.normal(size=(nz, ny, nx))
        Ap = np.zeros_like(p)
        L.ref_spmv(p.ctypes.data, Ap.ctypes.data)
        inv = np.zeros_like(p)
        L.ref_invm(inv.ctypes.data)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), dims=dims, h=h, bc=bc, p=p, Ap=Ap, invM=inv,
                            mask=mask if masked else np.zeros(0, np.uint8))
        manifest[name] = {"kind": "spmv", "dims": dims, "bc": bc, "masked": masked}

    # RHS build
    dims, h, bc = (6, 5, 4), (1 / 6, 1 / 5, 1 / 4), (P, P, P, P, N, N)
    nx, ny, nz = dims
    setup(L, dims, h, bc, None)
    u = rng.normal(size=(nz, ny, nx + 1))
    v = rng.normal(size=(nz, ny + 1, nx))
    w = rng.normal(size=(nz + 1, ny, nx))
    rhs = np.zeros((nz, ny, nx))
    L.ref_rhs(1.7, 0.3, u.ctypes.data, v.ctypes.data, w.ctypes.data, rhs.ctypes.data)
    np.savez_compressed(os.path.join(HERE, "rhs_ppn.npz"), dims=dims, h=h, bc=bc, u=u, v=v, w=w, rho_f=1.7, dt=0.3,
                        rhs=rhs)
    manifest["rhs_ppn"] = {"kind": "rhs", "dims": dims, "bc": bc}

    # solves: the C1 workload at full size (32^3, periodic, iid U[-1,1] minus mean)
    # and reduced masked / Neumann cases
    solve_cases = [
        ("solve_c1_32", (32, 32, 32), (P,) * 6, 0, 1e-10 * (1 / 32) / np.sqrt(6)),
        ("solve_ppn_spheres_20", (20, 20, 20), (P, P, P, P, N, N), 6, 1e-9),
        ("solve_nnn_spheres_16x12x10", (16, 12, 10), (N,) * 6, 2, 1e-12),
        ("solve_ppp_spheres_24", (24, 24, 24), (P,) * 6, 5, 1e-8),
    ]
    for name, dims, bc, nsph, resid in solve_cases:
        nx, ny, nz = dims
        h = (1 / nx, 1 / ny, 1 / nz)
        mask = None
        if nsph:
            cents = rng.random((nsph, 3))
            if bc[4] == N:
                cents[:, 2] = 0.25 + 0.5 * cents[:, 2]
            mask = spheres_mask(dims, h, bc, cents, np.full(nsph, 0.14))
        b = rng.uniform(-1, 1, (nz, ny, nx))
        if mask is not None:
            b[mask == 1] = 0
            b[mask == 0] -= b[mask == 0].mean()
        else:
            b -= b.mean()
        setup(L, dims, h, bc, mask)
        phi = np.zeros_like(b)
        it, rs = ctypes.c_int(), ctypes.c_double()
        L.ref_solve(b.ctypes.data, resid, 20000, phi.ctypes.data, ctypes.byref(it), ctypes.byref(rs))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), dims=dims, h=h, bc=bc, rhs=b, phi=phi,
                            mask=mask if mask is not None else np.zeros(0, np.uint8), pp_residual=resid,
                            niter=it.value, resid=rs.value)
        manifest[name] = {"kind": "solve", "dims": dims, "bc": bc, "pp_residual": resid, "niter": it.value,
                          "resid": rs.value, "solid_cells": int(mask.sum()) if mask is not None else 0}
        print(name, it.value, rs.value)
    # whole solves as the time loop calls them: rhs from u*, v*, w* (PP_rhs),
    # particle masking, coeffs_refine, PCG (cuda_PP_cg / cuda_PP_cg_noparts)
    dropin_cases = [
        ("dropin_ppn_spheres_20", (20, 18, 16), (P, P, P, P, N, N), 5, 1e-9),
        ("dropin_ppn_noparts_16", (16, 16, 12), (P, P, P, P, N, N), 0, 1e-10),
    ]
    for name, dims, bc, nsph, resid in dropin_cases:
        nx, ny, nz = dims
        h = (1 / nx, 1 / ny, 1 / nz)
        mask = None
        if nsph:
            cents = rng.random((nsph, 3))
            cents[:, 2] = 0.25 + 0.5 * cents[:, 2]
            mask = spheres_mask(dims, h, bc, cents, np.full(nsph, 0.15))
        u = rng.normal(size=(nz, ny, nx + 1))
        v = rng.normal(size=(nz, ny + 1, nx))
        w = rng.normal(size=(nz + 1, ny, nx))
        # periodic x, y: the face on the far side equals the first face;
        # Neumann z: no flow through the walls (a consistent rhs without spheres)
        u[:, :, nx] = u[:, :, 0]
        v[:, ny, :] = v[:, 0, :]
        w[0] = 0.0
        w[nz] = 0.0
        setup(L, dims, h, bc, mask)
        phi = np.zeros((nz, ny, nx))
        it, rs = ctypes.c_int(), ctypes.c_double()
        L.ref_solve_u(1.3, 0.01, u.ctypes.data, v.ctypes.data, w.ctypes.data, resid, 20000, phi.ctypes.data,
                      ctypes.byref(it), ctypes.byref(rs))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), dims=dims, h=h, bc=bc, u=u, v=v, w=w, rho_f=1.3,
                            dt=0.01, mask=mask if mask is not None else np.zeros(0, np.uint8), pp_residual=resid,
                            phi=phi, niter=it.value, resid=rs.value)
        manifest[name] = {"kind": "dropin", "dims": dims, "bc": bc, "pp_residual": resid, "niter": it.value,
                          "resid": rs.value}
        print(name, it.value, rs.value)
    # the time loop's steps after the solve: phi ghosts, projection, pressure update
    import layout
    epi_cases = [
        ("epilogue_ppn_spheres", (12, 10, 8), (P, P, P, P, N, N), 3),
        ("epilogue_nnp_noparts", (9, 11, 7), (N, N, N, N, P, P), 0),
    ]
    for name, dims, bc, nsph in epi_cases:
        nx, ny, nz = dims
        h = (1 / nx, 1.2 / ny, 0.9 / nz)
        mask = None
        if nsph:
            cents = rng.random((nsph, 3))
            cents[:, 2] = 0.25 + 0.5 * cents[:, 2]
            mask = spheres_mask(dims, h, bc, cents, np.full(nsph, 0.2))
        setup(L, dims, h, bc, mask)
        phi = rng.normal(size=(nz, ny, nx))
        us = rng.normal(size=(nz, ny, nx + 1))
        vs = rng.normal(size=(nz, ny + 1, nx))
        ws = rng.normal(size=(nz + 1, ny, nx))
        p0 = rng.normal(size=(nz, ny, nx))
        sz = np.zeros(4, np.int64)
        L.ref_sizes(sz.ctypes.data)
        ub, vb, wb = np.zeros(sz[1]), np.zeros(sz[2]), np.zeros(sz[3])
        phib, pb = np.zeros(sz[0]), np.zeros(sz[0])
        usb, vsb, wsb, p0b = layout.fx_to_s3b(us), layout.fy_to_s3b(vs), layout.fz_to_s3b(ws), layout.cells_to_s3b(p0)
        assert (usb.size, vsb.size, wsb.size, p0b.size) == tuple(int(v) for v in (sz[1], sz[2], sz[3], sz[0]))
        L.ref_epilogue(1.3, 0.02, 0.5, phi.ctypes.data, usb.ctypes.data, vsb.ctypes.data, wsb.ctypes.data,
                       p0b.ctypes.data, phib.ctypes.data, ub.ctypes.data, vb.ctypes.data, wb.ctypes.data,
                       pb.ctypes.data)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), dims=dims, h=h, bc=bc, rho_f=1.3, dt=0.02, nu=0.5,
                            mask=mask if mask is not None else np.zeros(0, np.uint8), phi=phi, us=us, vs=vs, ws=ws,
                            p0=p0, u=layout.fx_from_s3b(ub, dims), v=layout.fy_from_s3b(vb, dims),
                            w=layout.fz_from_s3b(wb, dims), p=layout.cells_from_s3b(pb, dims), phi_b=phib)
        manifest[name] = {"kind": "epilogue", "dims": dims, "bc": bc}
        print(name)
    json.dump(manifest, open(os.path.join(HERE, "manifest.json"), "w"), indent=1)


if __name__ == "__main__":
    main()
