"""Synthetic inputs of the measured workloads, generated on the oracle side.

TEST INFRASTRUCTURE ONLY.  The reference publishes no inputs for its pressure
solve, so every workload is drawn from seeds: sphere centres from the
reference's Ranq1 generator (src/rng.c:25-107, restated in the oracle's C
library), the solid mask by the oracle's restatement of build_phase
(src/particle_kernel.cu:148-253), right-hand sides as Gaussian random fields
with power spectrum k^(-11/3) for 1 <= |k| <= 32, evolved in Fourier space by an
Ornstein-Uhlenbeck process (correlation 0.95 per step).

The solver package draws the same inputs through its own library.  This module
restates that procedure on the oracle's generator so that the CPU arm of the
benchmark, which times the oracle, builds its inputs without loading the
solver's library; tests/test_pyproblems.py checks that both produce identical
arrays.
"""
import numpy as np

import pyoracle

PERIODIC, NEUMANN = 0, 2
# name -> (cells per side, boundary code x/y/z, spheres, radius in cells, seed, tolerance)
WORKLOADS = {
    "C1": (32, "ppp", 0, 0, 1, 1e-10),
    "C2": (128, "ppn", 64, 8, 2, 1e-10),
    "C3": (256, "ppn", 1000, 6, 3, 1e-8),
    "C4": (64, "ppn", 128, 4, 4, 1e-10),
    "C5": (512, "ppn", 4000, 5, 5, 1e-8),
}
SPECTRUM_KMAX = 32
OU_CORRELATION = 0.95


def grid(n, code):
    """Oracle grid on the unit cube; code 'ppn' = periodic x, y and Neumann z."""
    bc = []
    for ch in code:
        bc += [PERIODIC if ch == "p" else NEUMANN] * 2
    return pyoracle.grid(n, n, n, bc=tuple(bc))


def sphere_centres(g, count, radius_cells, seed):
    """Centres uniform in the box, accepted in order when no earlier sphere lies
    closer than two radii (minimum image along periodic axes); along a Neumann
    axis a centre keeps one radius from the walls.  Draws come in blocks of
    4096 triples, block b from the Ranq1 stream seeded seed * 1000003 + b."""
    if count == 0:
        return np.zeros((0, 3)), np.zeros(0)
    box = np.array([g.nx * g.dx, g.ny * g.dy, g.nz * g.dz])
    rad = radius_cells * g.dx
    periodic = np.array([g.bc[0] == PERIODIC, g.bc[2] == PERIODIC, g.bc[4] == PERIODIC])
    low = np.where(periodic, 0.0, rad)
    span = np.where(periodic, box, box - rad) - low
    accepted = []
    block = 0
    while len(accepted) < count:
        draws = pyoracle.rng_uniform(seed * 1_000_003 + block, 3 * 4096).reshape(4096, 3)
        block += 1
        for c in low + span * draws:
            if accepted:
                sep = np.asarray(accepted) - c
                sep = np.where(periodic, sep - box * np.round(sep / box), sep)
                if (np.einsum("ij,ij->i", sep, sep) < (2 * rad) ** 2).any():
                    continue
            accepted.append(c)
            if len(accepted) == count:
                break
        if block > 500:
            raise RuntimeError("sphere placement did not finish")
    return np.asarray(accepted), np.full(count, rad)


def _amplitude(shape):
    kz, ky, kx = [np.fft.fftfreq(m) * m for m in shape]
    kmag = np.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)
    amp = np.zeros(shape)
    band = (kmag >= 1) & (kmag <= SPECTRUM_KMAX)
    amp[band] = kmag[band] ** (-11.0 / 6.0)
    return amp


def _white(shape, seed):
    draws = pyoracle.rng_gauss(seed, 2 * int(np.prod(shape)))
    return (draws[0::2] + 1j * draws[1::2]).reshape(shape)


def _finish(spectrum, solid):
    """Real part of the field, unit RMS, zero on solid cells, zero mean on fluid."""
    f = np.real(np.fft.ifftn(spectrum)).astype(np.float64)
    f /= np.sqrt(np.mean(f * f))
    if solid is None:
        f -= f.mean()
    else:
        fluid = solid == 0
        f[~fluid] = 0.0
        f[fluid] -= f[fluid].mean()
    return np.ascontiguousarray(f)


class OUFields:
    """The right-hand side sequence: b_0 from white noise seeded seed * 7919,
    then b_{t+1}(k) = 0.95 b_t(k) + sqrt(1 - 0.95^2) S(k) xi_t(k) with xi_t
    seeded seed * 7919 + t + 1."""

    def __init__(self, shape, seed, solid):
        self.shape, self.seed, self.solid = shape, seed, solid
        self.amp = _amplitude(shape)
        self.t = 0
        self.spec = _white(shape, seed * 7919) * self.amp

    def current(self):
        return _finish(self.spec, self.solid)

    def advance(self):
        self.t += 1
        xi = _white(self.shape, self.seed * 7919 + self.t)
        self.spec = OU_CORRELATION * self.spec + np.sqrt(1 - OU_CORRELATION ** 2) * self.amp * xi
        return self.current()


def workload(name):
    """(oracle grid, solid mask or None, sphere centres, radii, seed, tol) of a named workload."""
    n, code, count, rad, seed, tol = WORKLOADS[name]
    g = grid(n, code)
    cents, radii = sphere_centres(g, count, rad, seed)
    solid = pyoracle.sphere_mask(g, cents, radii) if count else None
    return g, solid, cents, radii, seed, tol
