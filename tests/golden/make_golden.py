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
  cages_*.npz  particle centres and radii, and the phase, phase_shell and face
               flags cuda_build_cages builds from them (src/cuda_particle.cu:
               1516-1646 around the kernels of src/particle_kernel.cu:79-576)

Needs the reference tree; run:  python tests/golden/make_golden.py
(`--only cages` rewrites the cage fixtures alone.)
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
    L.ref_build_cages.argtypes = [ctypes.c_int, ctypes.c_int, v, v, v, v, v, v]
    L.ref_part_struct_bytes.restype = ctypes.c_longlong
    return L


def cage_particles(rng, dims, h, bc, count, rad_cells):
    """Centres uniform in the box (overlaps allowed: the last index wins a
    cell), plus, along periodic axes, the shifted copy of every particle within
    a cage of the boundary -- the ghost particles the host program hands the
    cage builder of a periodic one-rank domain."""
    ext = np.array(dims) * np.array(h)
    rows = []
    for _ in range(count):
        c = rng.random(3) * ext
        r = rad_cells * h[0] * (0.8 + 0.4 * rng.random())
        rows.append([c[0], c[1], c[2], r])
    ghosts = []
    for row in rows:
        for a in range(3):
            if bc[2 * a] == P:
                if row[a] < 2 * row[3]:
                    g = list(row)
                    g[a] += ext[a]
                    ghosts.append(g)
                elif row[a] > ext[a] - 2 * row[3]:
                    g = list(row)
                    g[a] -= ext[a]
                    ghosts.append(g)
    return np.array(rows + ghosts, np.float64).reshape(-1, 4)


def cages(L, manifest):
    """Fixtures of cuda_build_cages: seeded particle sets on small one-rank
    domains; radius 3 cells on an even grid gives cages of 8 cells, the case
    where the reference's launch reaches one cell short of its cage."""
    rng = np.random.default_rng(20261204)
    cases = [
        ("cages_ppn_16", (16, 14, 12), (P, P, P, P, N, N), 7, 2.4, 1),
        ("cages_nnn_odd", (15, 13, 11), (N,) * 6, 6, 2.0, 1),
        ("cages_ppp_r3", (20, 16, 18), (P,) * 6, 5, 3.0, 1),
        ("cages_pnp_mixed", (17, 12, 14), (P, P, N, N, P, P), 8, 1.6, 1),
        ("cages_nnp_noparts", (9, 11, 7), (N, N, N, N, P, P), 0, 0, 0),
    ]
    for name, dims, bc, count, rad, with_parts in cases:
        nx, ny, nz = dims
        h = (1 / nx, 1 / ny, 1 / nz)
        if name == "cages_ppp_r3":
            # exact radius of 3 cells (cage of 8 cells)
            parts = cage_particles(rng, dims, h, bc, count, rad)
            parts[:, 3] = 3 * h[0]
        else:
            parts = cage_particles(rng, dims, h, bc, count, rad)
        setup(L, dims, h, bc, None)
        sz = np.zeros(4, np.int64)
        L.ref_sizes(sz.ctypes.data)
        phase, shell = np.zeros(sz[0], np.int32), np.zeros(sz[0], np.int32)
        fu, fv, fw = np.zeros(sz[1], np.int32), np.zeros(sz[2], np.int32), np.zeros(sz[3], np.int32)
        parts = np.ascontiguousarray(parts)
        L.ref_build_cages(with_parts, len(parts), parts.ctypes.data if len(parts) else None, phase.ctypes.data,
                          shell.ctypes.data, fu.ctypes.data, fv.ctypes.data, fw.ctypes.data)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), dims=dims, h=h, bc=bc, with_parts=with_parts,
                            parts=parts, phase=phase, phase_shell=shell, flag_u=fu, flag_v=fv, flag_w=fw)
        manifest[name] = {"kind": "cages", "dims": dims, "bc": bc, "nparts": int(len(parts)),
                          "solid_cells": int((phase > -1).sum()) if with_parts else 0,
                          "shell_cells": int((shell == 0).sum()) if with_parts else 0,
                          "part_struct_bytes": int(L.ref_part_struct_bytes())}
        print(name, len(parts), manifest[name]["solid_cells"], manifest[name]["shell_cells"])


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
    if "--only" in sys.argv and sys.argv[sys.argv.index("--only") + 1] == "cages":
        manifest = json.load(open(os.path.join(HERE, "manifest.json")))
        cages(L, manifest)
        json.dump(manifest, open(os.path.join(HERE, "manifest.json"), "w"), indent=1)
        return
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
    cages(L, manifest)
    json.dump(manifest, open(os.path.join(HERE, "manifest.json"), "w"), indent=1)


if __name__ == "__main__":
    main()
