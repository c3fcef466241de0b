"""The algebra of the fused FP32 iteration (k1_fused in
bluebottle-3.0_gb300/csrc/bbpp_tma.cu), restated in FP64 numpy and checked
against classic Jacobi-PCG on the same SPD system.

The fused kernel of iteration q applies the update iteration q - 1 deferred
(r -= alpha Ap, x += alpha p), forms p_q = z + beta_q p_{q-1} with beta_q from
the one-step expansion
    (r_{q-1}, z_{q-1}) = (r_{q-2}, z_{q-2}) - 2 alpha (Ap, z) + alpha^2 (Ap, Ap / dL)
(the exact product, summed in the same kernel, restarts the expansion), and
ends iteration q - 1 with the exact products.  A checkpoint folds the pending
step into x and replaces r by the explicit residual.  In exact arithmetic the
iterates are classic PCG's; in FP64 they agree to round-off."""
import numpy as np
import pytest

sp = pytest.importorskip("scipy.sparse")


def laplacian(n, shift, seed):
    """A 3-D 7-point Laplacian on n^3 cells (Dirichlet walls) with a random
    positive diagonal shift, so that the Jacobi weights differ per cell."""
    one = sp.diags([-np.ones(n - 1), 2 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1])
    eye = sp.identity(n)
    a = sp.kron(sp.kron(one, eye), eye) + sp.kron(sp.kron(eye, one), eye) + sp.kron(sp.kron(eye, eye), one)
    rng = np.random.default_rng(seed)
    return (a + sp.diags(shift * rng.random(n ** 3))).tocsr()


def classic_pcg(a, b, iters, replace_every):
    dinv = 1.0 / a.diagonal()
    x = np.zeros_like(b)
    r = b.copy()
    z = dinv * r
    p = z.copy()
    rz = r @ z
    xs = []
    for q in range(1, iters + 1):
        ap = a @ p
        alpha = rz / (p @ ap)
        x = x + alpha * p
        r = r - alpha * ap
        if q % replace_every == 0:
            r = b - a @ x
        z = dinv * r
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
        xs.append(x.copy())
    return xs


def fused_pcg(a, b, iters, replace_every):
    """The fused form: kernel q of iters + 1 kernels; returns x after each
    completed iteration (settled at the end of the kernel that completes it)."""
    dinv = 1.0 / a.diagonal()
    x = np.zeros_like(b)
    r = b.copy()                 # the residual init kernel
    rz = r @ (dinv * r)
    first, lag = True, False
    alpha = beta = 0.0
    p_prev = ap_prev = None
    xs = []
    for q in range(1, iters + 2):
        # the deferred update of iteration q - 1
        if lag:
            r = r - alpha * ap_prev
            x = x + alpha * p_prev
        z = dinv * r
        p = z.copy() if first else z + beta * p_prev
        ap = a @ p
        pap, rz_exact, c1, c2 = p @ ap, r @ z, ap @ z, ap @ (dinv * ap)
        if lag:               # iteration q - 1 ends here, on a settled (x, r)
            xs.append(x.copy())
            rz = rz_exact
        alpha = rz / pap
        beta = (rz - 2.0 * alpha * c1 + alpha * alpha * c2) / rz
        first, lag = False, True
        p_prev, ap_prev = p, ap
        if q % replace_every == 0 and q <= iters:
            # checkpoint: fold the pending step, replace r, exact beta
            x = x + alpha * p_prev
            r = b - a @ x
            rz_new = r @ (dinv * r)
            beta = rz_new / rz
            rz = rz_new
            lag = False
            xs.append(x.copy())
    return xs[:iters]


@pytest.mark.parametrize("n,shift,replace_every", [(6, 0.1, 50), (8, 0.01, 20), (5, 1.0, 7)])
def test_fused_iteration_is_pcg(n, shift, replace_every):
    a = laplacian(n, shift, seed=n)
    rng = np.random.default_rng(n + 1)
    b = rng.standard_normal(n ** 3)
    iters = 60
    xc = classic_pcg(a, b, iters, replace_every)
    xf = fused_pcg(a, b, iters, replace_every)
    assert len(xf) == iters
    for q in range(iters):
        scale = np.abs(xc[q]).max()
        assert np.abs(xf[q] - xc[q]).max() <= 1e-9 * scale, q
    # and it converges like PCG
    res = np.linalg.norm(b - a @ xf[-1]) / np.linalg.norm(b)
    assert res < 1e-6


def test_expansion_matches_direct_product():
    """Restarted from the exact product every step, the one-step expansion of
    (r, z) matches the directly summed product to round-off."""
    a = laplacian(6, 0.05, seed=3)
    b = np.random.default_rng(4).standard_normal(6 ** 3)
    dinv = 1.0 / a.diagonal()
    r = b.copy()
    z = dinv * r
    p = z.copy()
    rz = r @ z
    for _ in range(30):
        ap = a @ p
        alpha = rz / (p @ ap)
        est = rz - 2.0 * alpha * (ap @ z) + alpha * alpha * (ap @ (dinv * ap))
        r = r - alpha * ap
        z = dinv * r
        exact = r @ z
        assert abs(est - exact) <= 1e-10 * abs(rz)
        p = z + (exact / rz) * p
        rz = exact
