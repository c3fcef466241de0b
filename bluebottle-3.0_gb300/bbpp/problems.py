"""Seeded synthetic pressure-Poisson problems.

The reference publishes no dataset or benchmark inputs for this path; these
generators produce inputs with the shapes, boundary conditions, sphere counts
and RHS spectra of the five workloads the solver is measured on:

  C1  32^3, periodic xyz, no spheres, RHS iid U[-1,1] minus its mean, tol 1e-10
  C2  128^3, periodic xy / Neumann z, 64 spheres r = 8 cells, spectral RHS, tol 1e-10
  C3  256^3, periodic xy / Neumann z, 1000 spheres r = 6 cells, spectral RHS, tol 1e-8
  C4  64^3 training set (128 spheres r = 4, OU-evolved spectral RHS); evaluation at 256^3
  C5  512^3, periodic xy / Neumann z, 4000 spheres r = 5, 50 OU-evolved solves

Domain [0,1]^3 so dx = 1/n.  Random numbers come from the reference's Ranq1
generator (src/rng.c:25-107) through the library's host code, so the streams
are reproducible in C and Python.
"""
import numpy as np

from . import NEUMANN, PERIODIC, Grid, rng_gauss, rng_uniform

CONFIGS = {
    "C1": dict(n=32, bc="ppp", nsph=0, rad=0, rhs="uniform", tol=1e-10, seed=1),
    "C2": dict(n=128, bc="ppn", nsph=64, rad=8, rhs="spectral", tol=1e-10, seed=2),
    "C3": dict(n=256, bc="ppn", nsph=1000, rad=6, rhs="spectral", tol=1e-8, seed=3),
    "C4": dict(n=64, bc="ppn", nsph=128, rad=4, rhs="spectral", tol=1e-10, seed=4),
    "C5": dict(n=512, bc="ppn", nsph=4000, rad=5, rhs="spectral", tol=1e-8, seed=5),
}

KMAX = 32          # spectral RHS: power spectrum k^(-11/3) for 1 <= |k| <= 32
OU_RHO = 0.95      # OU correlation per step


def bc_tuple(code):
    """'ppn' -> (W,E,S,N,B,T) with periodic x, y and Neumann z."""
    m = {"p": PERIODIC, "n": NEUMANN}
    return (m[code[0]],) * 2 + (m[code[1]],) * 2 + (m[code[2]],) * 2


def make_grid(n, bc="ppn", ny=None, nz=None):
    ny = n if ny is None else ny
    nz = n if nz is None else nz
    return Grid.make(n, ny, nz, 1.0 / n, 1.0 / ny, 1.0 / nz, bc_tuple(bc))


def place_spheres(grid, nsph, rad_cells, seed, max_tries=2_000_000):
    """Non-overlapping spheres (|ci - cj| >= 2r, minimum image in periodic
    directions) with centres uniform in the box; in a Neumann direction the
    centre stays at least r from the walls so spheres do not cut them.
    Returns (centres (nsph,3), radii (nsph,))."""
    if nsph == 0:
        return np.zeros((0, 3)), np.zeros(0)
    L = np.array([grid.nx * grid.dx, grid.ny * grid.dy, grid.nz * grid.dz])
    r = rad_cells * grid.dx
    per = np.array([grid.bc[0] == PERIODIC, grid.bc[2] == PERIODIC, grid.bc[4] == PERIODIC])
    lo = np.where(per, 0.0, r)
    hi = np.where(per, L, L - r)
    batch = 4096
    cents = np.zeros((nsph, 3))
    k = 0
    tries = 0
    stream = 0
    while k < nsph:
        u = rng_uniform(seed * 1_000_003 + stream, 3 * batch).reshape(batch, 3)
        stream += 1
        cand = lo + (hi - lo) * u
        for c in cand:
            tries += 1
            if tries > max_tries:
                raise RuntimeError("could not place %d spheres" % nsph)
            if k:
                d = cents[:k] - c
                d = np.where(per, d - L * np.round(d / L), d)
                if np.any(np.einsum("ij,ij->i", d, d) < (2 * r) ** 2):
                    continue
            cents[k] = c
            k += 1
            if k == nsph:
                break
    return cents, np.full(nsph, r)


def sphere_mask_host(grid, cents, radii):
    """Host mask with the same arithmetic as the device builder (used only for
    inputs; the oracle has its own restatement)."""
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    m = np.zeros((nz, ny, nx), np.uint8)
    per = (grid.bc[0] == PERIODIC, grid.bc[2] == PERIODIC, grid.bc[4] == PERIODIC)
    L = (nx * grid.dx, ny * grid.dy, nz * grid.dz)
    d = (grid.dx, grid.dy, grid.dz)
    n = (nx, ny, nz)
    for (cx, cy, cz), r in zip(cents, radii):
        irad = 1.0 / r
        for ox in ((-1, 0, 1) if per[0] else (0,)):
            for oy in ((-1, 0, 1) if per[1] else (0,)):
                for oz in ((-1, 0, 1) if per[2] else (0,)):
                    C = (cx + ox * L[0], cy + oy * L[1], cz + oz * L[2])
                    rng = []
                    for a in range(3):
                        i0 = max(int(np.floor((C[a] - r) / d[a])) - 1, 0)
                        i1 = min(int(np.ceil((C[a] + r) / d[a])) + 1, n[a] - 1)
                        rng.append((i0, i1))
                    if any(i1 < i0 for i0, i1 in rng):
                        continue
                    ii = np.arange(rng[0][0], rng[0][1] + 1)
                    jj = np.arange(rng[1][0], rng[1][1] + 1)
                    kk = np.arange(rng[2][0], rng[2][1] + 1)
                    xx = ((ii + 1).astype(np.float64) - 0.5) * d[0] - C[0]
                    yy = ((jj + 1).astype(np.float64) - 0.5) * d[1] - C[1]
                    zz = ((kk + 1).astype(np.float64) - 0.5) * d[2] - C[2]
                    d2 = (xx[None, None, :] * xx[None, None, :] + yy[None, :, None] * yy[None, :, None]) \
                        + zz[:, None, None] * zz[:, None, None]
                    inside = np.floor(np.sqrt(d2) * irad) < 1
                    sub = m[kk[0]:kk[-1] + 1, jj[0]:jj[-1] + 1, ii[0]:ii[-1] + 1]
                    sub |= inside.astype(np.uint8)
    return m


def spectrum_amp(shape):
    """Amplitude sqrt(P(k)) = |k|^(-11/6) for 1 <= |k| <= KMAX, else 0."""
    nz, ny, nx = shape
    kz = np.fft.fftfreq(nz) * nz
    ky = np.fft.fftfreq(ny) * ny
    kx = np.fft.fftfreq(nx) * nx
    k2 = kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2
    k = np.sqrt(k2)
    amp = np.zeros(shape)
    sel = (k >= 1) & (k <= KMAX)
    amp[sel] = k[sel] ** (-11.0 / 6.0)
    return amp


def complex_noise(shape, seed):
    g = rng_gauss(seed, 2 * int(np.prod(shape)))
    return (g[0::2] + 1j * g[1::2]).reshape(shape)


def project_rhs(field, mask):
    """Unit RMS, zero on solid cells, zero mean over the fluid cells."""
    f = np.real(field).astype(np.float64)
    f /= np.sqrt(np.mean(f * f))
    if mask is not None:
        fluid = mask == 0
        f[~fluid] = 0.0
        f[fluid] -= f[fluid].mean()
    else:
        f -= f.mean()
    return np.ascontiguousarray(f)


def spectral_rhs(shape, seed, mask=None):
    amp = spectrum_amp(shape)
    field = np.fft.ifftn(complex_noise(shape, seed) * amp)
    return project_rhs(field, mask)


def uniform_rhs(shape, seed):
    f = rng_uniform(seed, int(np.prod(shape)), -1.0, 1.0).reshape(shape)
    return np.ascontiguousarray(f - f.mean())


class OUSequence:
    """RHS fields evolved by an Ornstein-Uhlenbeck process in Fourier space:
    b_{t+1}(k) = rho b_t(k) + sqrt(1 - rho^2) S(k) xi_t(k)."""

    def __init__(self, shape, seed, mask=None, rho=OU_RHO):
        self.shape, self.seed, self.mask, self.rho = shape, seed, mask, rho
        self.amp = spectrum_amp(shape)
        self.t = 0
        self.hat = complex_noise(shape, seed * 7919 + 0) * self.amp

    def field(self):
        return project_rhs(np.fft.ifftn(self.hat), self.mask)

    def step(self):
        self.t += 1
        xi = complex_noise(self.shape, self.seed * 7919 + self.t)
        self.hat = self.rho * self.hat + np.sqrt(1 - self.rho ** 2) * self.amp * xi
        return self.field()


def make_problem(name, n=None, seed=None, with_mask=True):
    """(grid, mask or None, rhs, tol) for a named workload; n overrides the size
    for reduced test cases (sphere radius and count scale with n)."""
    c = dict(CONFIGS[name])
    nn = c["n"] if n is None else n
    sd = c["seed"] if seed is None else seed
    grid = make_grid(nn, c["bc"])
    mask = None
    if c["nsph"] and with_mask:
        scale = nn / c["n"]
        nsph = max(1, int(round(c["nsph"] * scale ** 3)))
        rad = max(1.5, c["rad"] * scale)
        cents, radii = place_spheres(grid, nsph, rad, sd)
        mask = sphere_mask_host(grid, cents, radii)
    shape = grid.shape
    if c["rhs"] == "uniform":
        rhs = uniform_rhs(shape, sd)
    else:
        rhs = spectral_rhs(shape, sd, mask)
    return grid, mask, rhs, c["tol"]


class OUSequenceDevice:
    """The same Ornstein-Uhlenbeck right-hand-side sequence generated on the GPU
    (torch tensors, cuFFT), for grids where the host generator's FFTs and
    sequential Ranq1 draws would take minutes per field (the 512^3 workload).
    Same spectrum, correlation and projection as OUSequence; the white noise
    comes from torch's seeded CUDA generator instead of Ranq1, so the fields
    are a different draw of the same process.  Fields are float64 CUDA tensors
    of the grid's shape (z, y, x); mask is a (z, y, x) uint8 array (1 = solid)
    or None."""

    def __init__(self, shape, seed, mask=None, rho=OU_RHO, device="cuda"):
        import torch
        self.torch = torch
        self.shape, self.rho, self.device = tuple(shape), rho, device
        self.gen = torch.Generator(device=device)
        self.gen.manual_seed(int(seed) * 7919)
        nz, ny, nx = self.shape
        k = [torch.fft.fftfreq(m, d=1.0 / m, dtype=torch.float64, device=device) for m in (nz, ny, nx)]
        kmag = torch.sqrt(k[0][:, None, None] ** 2 + k[1][None, :, None] ** 2 + k[2][None, None, :] ** 2)
        band = (kmag >= 1) & (kmag <= KMAX)
        self.amp = torch.where(band, kmag.clamp(min=1.0) ** (-11.0 / 6.0), torch.zeros_like(kmag))
        del kmag, band
        self.fluid = None
        if mask is not None:
            self.fluid = torch.as_tensor(np.ascontiguousarray(mask)).to(device) == 0
        self.t = 0
        self.hat = self._noise() * self.amp

    def _noise(self):
        torch = self.torch
        re = torch.randn(self.shape, generator=self.gen, dtype=torch.float64, device=self.device)
        im = torch.randn(self.shape, generator=self.gen, dtype=torch.float64, device=self.device)
        return torch.complex(re, im)

    def field(self):
        """The current field: real part, unit RMS, zero on solid cells, zero mean on fluid cells."""
        torch = self.torch
        f = torch.fft.ifftn(self.hat).real.contiguous()
        f /= torch.sqrt(torch.mean(f * f))
        if self.fluid is None:
            f -= f.mean()
        else:
            f.masked_fill_(~self.fluid, 0.0)
            f -= self.fluid * (f.sum() / self.fluid.sum())
        return f

    def step(self):
        self.t += 1
        xi = self._noise()
        xi *= self.amp
        self.hat.mul_(self.rho).add_(xi, alpha=float(np.sqrt(1 - self.rho ** 2)))
        return self.field()
