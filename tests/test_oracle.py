"""CPU tests of the oracle: operator identities and known answers.

The operator is the reference's (-A) (src/solver_kernel.cu:684-707, :824-829)
and the method its Jacobi PCG (src/cuda_solver.cu:150-279).
"""
import itertools

import numpy as np
import pytest

P, N = 0, 2


def dense(orc, g, mask=None):
    n = g.nx * g.ny * g.nz
    A = np.zeros((n, n))
    e = np.zeros((g.nz, g.ny, g.nx))
    for c in range(n):
        e.flat[:] = 0
        e.flat[c] = 1
        A[:, c] = orc.spmv(g, e, mask).ravel()
    return A


@pytest.mark.parametrize("bc", [(P,) * 6, (P, P, P, P, N, N), (N,) * 6])
def test_spmv_symmetric(orc, bc):
    g = orc.grid(5, 4, 6, bc=bc)
    A = dense(orc, g)
    assert np.allclose(A, A.T, rtol=0, atol=1e-9 * np.abs(A).max())
    w = np.linalg.eigvalsh(A)
    assert w.min() > -1e-8 * w.max()


def test_periodic_eigen_kat(orc):
    """Discrete Fourier modes are exact eigenvectors of the periodic operator:
    lambda_k = sum_d (4/h_d^2) sin^2(pi k_d / n_d)."""
    nx, ny, nz = 8, 6, 10
    g = orc.grid(nx, ny, nz, bc=(P,) * 6)
    for kx, ky, kz in [(1, 0, 0), (2, 3, 1), (4, 3, 5), (0, 0, 0)]:
        z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        v = np.cos(2 * np.pi * (kx * x / nx + ky * y / ny + kz * z / nz))
        lam = (4 * nx ** 2 * np.sin(np.pi * kx / nx) ** 2 + 4 * ny ** 2 * np.sin(np.pi * ky / ny) ** 2
               + 4 * nz ** 2 * np.sin(np.pi * kz / nz) ** 2)
        assert np.allclose(orc.spmv(g, v), lam * v, rtol=1e-12, atol=1e-9 * max(lam, 1))


def test_neumann_row_sums_zero(orc):
    g = orc.grid(6, 5, 7, bc=(N,) * 6)
    assert np.abs(orc.spmv(g, np.ones((7, 5, 6)))).max() < 1e-9


def test_solid_rows_identity_like(orc):
    g = orc.grid(6, 6, 6, bc=(P, P, P, P, N, N))
    mask = np.zeros((6, 6, 6), np.uint8)
    mask[2:4, 2:4, 2:4] = 1
    A = dense(orc, g, mask)
    m = mask.ravel().astype(bool)
    # solid row: only the diagonal, = -(sum of face flags)/6 (src/solver_kernel.cu:684-689)
    sub = A[m]
    diag = sub[np.arange(m.sum()), np.where(m)[0]]
    assert np.allclose(diag, -1.0, atol=1e-12)
    sub[np.arange(m.sum()), np.where(m)[0]] = 0
    assert np.abs(sub).max() == 0
    # fluid rows never couple to solid cells, and stay symmetric on the fluid set
    F = A[np.ix_(~m, ~m)]
    assert np.abs(A[np.ix_(~m, m)]).max() == 0
    assert np.allclose(F, F.T, atol=1e-9 * np.abs(F).max())


@pytest.mark.parametrize("bc,seed", [((P,) * 6, 1), ((P, P, P, P, N, N), 2), ((N,) * 6, 3), ((P, P, N, N, P, P), 4)])
def test_fluid_block_positive_semidefinite(orc, bc, seed):
    """(-A) restricted to the fluid cells is symmetric positive semi-definite for
    any solid set, including solids on the periodic seams and the walls; its
    solid rows stay decoupled.  Positive semi-definiteness on the fluid subspace
    is what the PCG relies on."""
    g = orc.grid(6, 5, 4, bc=bc)
    rng = np.random.default_rng(seed)
    mask = (rng.random((4, 5, 6)) < 0.25).astype(np.uint8)
    mask[0, 0, :] = 1  # a row of solids along a seam / wall
    A = dense(orc, g, mask)
    m = mask.ravel().astype(bool)
    F = A[np.ix_(~m, ~m)]
    assert np.allclose(F, F.T, rtol=0, atol=1e-9 * np.abs(F).max())
    w = np.linalg.eigvalsh(0.5 * (F + F.T))
    assert w.min() > -1e-9 * w.max()
    assert np.abs(A[np.ix_(~m, m)]).max() == 0 and np.abs(A[np.ix_(m, ~m)]).max() == 0


def test_invm_matches_diag(orc):
    g = orc.grid(5, 4, 6, bc=(P, P, N, N, N, N))
    A = dense(orc, g)
    assert np.allclose(orc.invm(g).ravel(), 1.0 / np.diag(A), rtol=1e-14)


def test_pcg_solves_dense(orc):
    g = orc.grid(6, 5, 4, bc=(P, P, P, P, N, N))
    mask = np.zeros((4, 5, 6), np.uint8)
    mask[1, 2, 3] = mask[2, 2, 3] = 1
    rng = np.random.default_rng(0)
    b = rng.uniform(-1, 1, (4, 5, 6))
    b[mask == 1] = 0
    b[mask == 0] -= b[mask == 0].mean()
    x, res = orc.pcg(g, b, mask, tol=1e-12)
    assert res["status"] == 0 and res["true_rel"] < 1e-12
    A = dense(orc, g, mask)
    f = mask.ravel() == 0
    xs = np.linalg.lstsq(A[np.ix_(f, f)], b.ravel()[f], rcond=None)[0]
    assert np.allclose(x.ravel()[f], xs, rtol=0, atol=1e-10 * np.abs(xs).max())
    assert np.all(x[mask == 1] == 0)


def test_pcg_ref_rule_and_tiny_rhs(orc):
    g = orc.grid(8, 8, 8)
    x, res = orc.pcg(g, np.zeros((8, 8, 8)), stop=0, tol=1e-6)
    assert res["status"] == 1 and res["iters"] == 0
    b = np.cos(2 * np.pi * np.arange(8) / 8)[None, None, :] * np.ones((8, 8, 8))
    x, res = orc.pcg(g, b, stop=0, tol=1e-8)
    # (r,z) <= tol^2 (b,b) with z = invM r
    assert res["status"] == 0 and res["rz"] <= 1e-16 * res["bb"]


def test_pcg_max_iter(orc):
    g = orc.grid(16, 16, 16)
    b = np.random.default_rng(1).uniform(-1, 1, (16, 16, 16))
    b -= b.mean()
    x, res = orc.pcg(g, b, tol=1e-14, max_iter=3)
    assert res["status"] == 2 and res["iters"] == 4


def test_sphere_mask_matches_bruteforce(orc):
    g = orc.grid(20, 18, 16, bc=(P, P, P, P, N, N))
    cents = np.array([[0.02, 0.5, 0.5], [0.7, 0.97, 0.3]])
    radii = np.array([0.15, 0.12])
    m = orc.sphere_mask(g, cents, radii)
    z, y, x = np.meshgrid(np.arange(16), np.arange(18), np.arange(20), indexing="ij")
    X, Y, Z = (x + 0.5) / 20, (y + 0.5) / 18, (z + 0.5) / 16
    ref = np.zeros_like(m)
    for (cx, cy, cz), r in zip(cents, radii):
        dx = X - cx
        dx -= np.round(dx)
        dy = Y - cy
        dy -= np.round(dy)
        ref |= (np.sqrt(dx * dx + dy * dy + (Z - cz) ** 2) < r).astype(np.uint8)
    assert np.array_equal(m, ref)


def test_rhs_div_and_refine(orc):
    g = orc.grid(4, 3, 5, bc=(P, P, P, P, N, N))
    rng = np.random.default_rng(3)
    u = rng.normal(size=(5, 3, 5))
    v = rng.normal(size=(5, 4, 4))
    w = rng.normal(size=(6, 3, 4))
    rhs = orc.rhs_div(g, 2.0, 0.5, u, v, w)
    div = (np.diff(u, axis=2) * 4 + np.diff(v, axis=1) * 3 + np.diff(w, axis=0) * 5)
    assert np.allclose(rhs, -4.0 * div, rtol=1e-13)
    mask = np.zeros((5, 3, 4), np.uint8)
    mask[2, 1, 1] = 1
    out = orc.rhs_mask_refine(g, mask, rhs)
    assert out[2, 1, 1] == 0
    keep = np.ones_like(mask, bool)
    keep[2, 1, 1] = False
    assert np.array_equal(out[keep], rhs[keep])
