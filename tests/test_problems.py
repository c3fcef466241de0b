"""CPU checks of the seeded synthetic workloads (bluebottle-3.0_gb300/bbpp/problems.py)
that the parity tests and the bench solve: sphere placement and masks, the
spectral and uniform right-hand sides, the Ornstein-Uhlenbeck sequence of the
learned guess, and the reduced-size problems."""
import numpy as np
import pytest

from bbpp import problems


def test_spheres_do_not_overlap_and_stay_off_the_walls(bbpp_lib):
    g = problems.make_grid(32, "ppn")
    cents, radii = problems.place_spheres(g, 40, 3, seed=11)
    r = 3 * g.dx
    assert cents.shape == (40, 3) and np.all(radii == r)
    # periodic x, y: anywhere in [0, 1); Neumann z: at least r from both walls
    assert np.all((cents[:, :2] >= 0) & (cents[:, :2] < 1))
    assert np.all((cents[:, 2] >= r) & (cents[:, 2] <= 1 - r))
    d = cents[:, None, :] - cents[None, :, :]
    d[..., :2] -= np.round(d[..., :2])  # minimum image in x, y
    dist = np.sqrt((d ** 2).sum(-1)) + np.eye(40) * 10
    assert dist.min() >= 2 * r
    # the same seed gives the same layout
    again, _ = problems.place_spheres(g, 40, 3, seed=11)
    assert np.array_equal(cents, again)


@pytest.mark.parametrize("bc", ["ppn", "nnn", "ppp"])
def test_sphere_mask_matches_brute_force(bbpp_lib, bc):
    """Cells whose centre lies strictly inside a sphere (or a periodic image of
    it), by the mask builder's bounding boxes against every cell."""
    g = problems.make_grid(24, bc, ny=20, nz=16)
    cents, radii = problems.place_spheres(g, 6, 3.5, seed=5)
    got = problems.sphere_mask_host(g, cents, radii)
    nz, ny, nx = g.shape
    zc = (np.arange(nz) + 0.5) * g.dz
    yc = (np.arange(ny) + 0.5) * g.dy
    xc = (np.arange(nx) + 0.5) * g.dx
    per = [bc[0] == "p", bc[1] == "p", bc[2] == "p"]
    want = np.zeros(g.shape, np.uint8)
    for (cx, cy, cz), r in zip(cents, radii):
        for ox in ((-1, 0, 1) if per[0] else (0,)):
            for oy in ((-1, 0, 1) if per[1] else (0,)):
                for oz in ((-1, 0, 1) if per[2] else (0,)):
                    dx = xc[None, None, :] - (cx + ox * nx * g.dx)
                    dy = yc[None, :, None] - (cy + oy * ny * g.dy)
                    dz = zc[:, None, None] - (cz + oz * nz * g.dz)
                    d2 = (dx * dx + dy * dy) + dz * dz
                    want |= (np.floor(np.sqrt(d2) * (1.0 / r)) < 1).astype(np.uint8)
    assert want.any()
    assert np.array_equal(got, want)


def test_spectral_rhs_band_and_projection(bbpp_lib):
    shape = (32, 32, 32)
    f = problems.spectral_rhs(shape, seed=3)
    # unit RMS, zero mean, and no energy outside 1 <= |k| <= 32
    assert abs(np.sqrt(np.mean(f * f)) - 1) < 1e-12 and abs(f.mean()) < 1e-14
    F = np.abs(np.fft.fftn(f)) ** 2
    outside = problems.spectrum_amp(shape) == 0
    assert F[outside].sum() <= 1e-20 * F.sum()
    # with a mask: zero on solid cells, zero mean over the fluid
    mask = np.zeros(shape, np.uint8)
    mask[4:9, 10:15, 2:30] = 1
    fm = problems.spectral_rhs(shape, seed=3, mask=mask)
    assert not fm[mask == 1].any()
    assert abs(fm[mask == 0].mean()) < 1e-14
    assert np.array_equal(fm, problems.spectral_rhs(shape, seed=3, mask=mask))


def test_ou_sequence_is_correlated_and_stationary(bbpp_lib):
    """b_{t+1}(k) = rho b_t(k) + sqrt(1 - rho^2) S(k) xi_t(k): successive fields
    correlate by rho, and the energy stays put."""
    seq = problems.OUSequence((32, 32, 32), seed=9)
    h0 = seq.hat.copy()
    seq.step()
    h1 = seq.hat.copy()
    corr = np.real(np.vdot(h0, h1)) / (np.linalg.norm(h0) * np.linalg.norm(h1))
    assert abs(corr - problems.OU_RHO) < 0.02
    e = [np.linalg.norm(h0)]
    for _ in range(20):
        seq.step()
        e.append(np.linalg.norm(seq.hat))
    assert max(e) / min(e) < 1.15
    # the fields it hands out are projected like any spectral right-hand side
    f = seq.field()
    assert abs(np.sqrt(np.mean(f * f)) - 1) < 1e-12


def test_uniform_rhs(bbpp_lib):
    f = problems.uniform_rhs((8, 8, 8), seed=1)
    assert abs(f.mean()) < 1e-15
    m = f + (problems.rng_uniform(1, 512, -1.0, 1.0).mean())
    assert m.min() >= -1 and m.max() <= 1
    assert np.array_equal(f, problems.uniform_rhs((8, 8, 8), seed=1))


@pytest.mark.parametrize("name,n", [("C1", 16), ("C2", 32), ("C3", 32)])
def test_reduced_problems(bbpp_lib, name, n):
    g, mask, rhs, tol = problems.make_problem(name, n=n)
    c = problems.CONFIGS[name]
    assert g.shape == (n, n, n) and tol == c["tol"]
    assert abs(rhs.mean() if mask is None else rhs[mask == 0].mean()) < 1e-13
    if c["nsph"]:
        assert mask is not None and mask.any() and not mask.all()
        assert not rhs[mask == 1].any()
    else:
        assert mask is None
