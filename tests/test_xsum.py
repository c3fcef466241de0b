"""The FP64 search kernel's exact neighbour sum (xsum6 in
bluebottle-3.0_gb300/csrc/bbpp_fast.cuh).

The plain FP64 iteration adds each interior cell's six neighbours as one
fixed-point sum on the integer pipe instead of five FP64 adds.  `model` below
restates that arithmetic with Python integers.  The CPU tests hold the model to
its stated bound against exact rational sums, compare it with the FP64 adds it
replaces, and hold the same C++ compiled for the host bit-exact to it; the GPU
tests hold the library's kernel bit-exact to the model and run whole solves
with the sum on and off.
"""
import os
import struct
import sys
from fractions import Fraction

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "bluebottle-3.0_gb300"))


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _float(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def fp64_adds(v):
    """The stencil's FP64 order: ((e + w) + (n + s)) + (t + b)."""
    return ((v[0] + v[1]) + (v[2] + v[3])) + (v[4] + v[5])


def model(v):
    """(sum, E): the kernel's result for six doubles and the largest biased
    exponent E it aligned to (None where it falls back to FP64 adds)."""
    bits = [_bits(float(x)) for x in v]
    E = max([1] + [(b >> 52) & 0x7FF for b in bits])
    if E < 128 or E > 2040:
        return fp64_adds([float(x) for x in v]), None
    acc = 0
    for b in bits:
        e = (b >> 52) & 0x7FF
        M = (b & ((1 << 52) - 1)) | ((1 << 52) if e else 0)
        w = (M << 11) >> min(E - max(e, 1) + 4, 63)
        acc += -w if b >> 63 else w
    assert abs(acc) < 1 << 63
    if acc == 0:
        return 0.0, E
    m = abs(acc)
    lz = 64 - m.bit_length()
    m <<= lz
    mant, rest = m >> 11, m & 0x7FF
    up = 1 if rest > 0x400 or (rest == 0x400 and mant & 1) else 0
    out = ((E + 3 - lz) << 52) + mant + up
    if acc < 0:
        out |= 1 << 63
    return _float(out), E


def sample(n, seed):
    """Six-tuples of the kinds a pressure iterate holds: smooth neighbourhoods
    (values within a few per cent of each other), magnitudes spread over 2^+-40,
    cancelling pairs, exact zeros (solid neighbours), a few subnormals and
    huge values, mixed signs."""
    rng = np.random.default_rng(seed)
    v = np.empty((n, 6))
    kind = rng.integers(0, 6, n)
    base = rng.standard_normal(n)[:, None]
    v[:] = base * (1 + 0.03 * rng.standard_normal((n, 6)))                             # 0: smooth
    spread = rng.standard_normal((n, 6)) * np.exp2(rng.integers(-40, 41, (n, 6)))
    v[kind == 1] = spread[kind == 1]                                                   # 1: wide exponents
    canc = base * (1 + 1e-9 * rng.standard_normal((n, 6)))
    canc[:, 1::2] *= -1
    v[kind == 2] = canc[kind == 2]                                                     # 2: cancellation
    z = v.copy()
    z[rng.random((n, 6)) < 0.5] = 0.0
    v[kind == 3] = z[kind == 3]                                                        # 3: solid neighbours
    v[kind == 4] = (rng.standard_normal((n, 6)) * 1e-310)[kind == 4]                   # 4: subnormal (fallback)
    v[kind == 5] = (rng.standard_normal((n, 6)) * np.exp2(rng.integers(-1000, 1000, (n, 1))))[kind == 5]
    return v


def test_model_within_bound_of_exact_sum():
    """Within 1/2 ulp of the result plus six units of 2^(E - 1082) (ulp(max)/128)
    of the exact sum, for every sample that takes the integer path."""
    v = sample(4000, 1)
    n_int = 0
    for row in v:
        got, E = model(row)
        exact = sum(Fraction(float(x)) for x in row)
        if E is None:
            assert got == fp64_adds(list(row))
            continue
        n_int += 1
        bound = Fraction(abs(np.spacing(got))) / 2 + 6 * Fraction(2) ** (E - 1082)
        assert abs(Fraction(got) - exact) <= bound, (row, got, float(exact))
    assert n_int > 3000


def test_model_no_less_accurate_than_fp64_adds():
    """Against the exact sum the integer path is correctly rounded at least as
    often as the five FP64 adds, and never much further off."""
    v = sample(4000, 2)
    ok_int = ok_fp = 0
    worse = 0
    for row in v:
        got, E = model(row)
        if E is None:
            continue
        exact = sum(Fraction(float(x)) for x in row)
        rn = float(exact)  # correctly rounded
        fp = fp64_adds(list(row))
        ok_int += got == rn
        ok_fp += fp == rn
        scale = max(abs(float(x)) for x in row)
        if abs(Fraction(got) - exact) > abs(Fraction(fp) - exact) + Fraction(scale) * Fraction(2) ** -58:
            worse += 1
    assert ok_int >= ok_fp and ok_int > 0.95 * 3000
    assert worse == 0


def test_model_edge_cases():
    one = 1.0
    assert model([one, 0, 0, 0, 0, 0]) == (1.0, 1023)
    assert model([1.0, -1.0, 2.0, -2.0, 0.5, -0.5])[0] == 0.0
    assert model([0.0] * 6)[1] is None                    # all zero: FP64 adds
    assert model([-0.0] * 6)[0] == 0.0 and np.signbit(model([-0.0] * 6)[0])
    s, E = model([1.0, 2.0 ** -60, 0, 0, 0, 0])           # far below ulp(max)/128: dropped
    assert E == 1023 and s == 1.0
    s, E = model([1.0, 2.0 ** -53, 2.0 ** -53, 0, 0, 0])  # 2 ulp/2 parts add exactly
    assert s == 1.0 + 2.0 ** -52
    assert model([1.0 + 2.0 ** -52, 2.0 ** -53, 0, 0, 0, 0])[0] == 1.0 + 2.0 ** -51  # tie to even
    assert np.isnan(model([np.inf, -np.inf, 0, 0, 0, 0])[0])
    assert model([np.inf, 1.0, 0, 0, 0, 0])[0] == np.inf
    big = 2.0 ** 1000
    assert model([big] * 6) == (6 * big, 2023)


EDGE_ROWS = [[1.0, 0, 0, 0, 0, 0], [0.0] * 6, [-0.0] * 6, [np.inf, 1, 0, 0, 0, 0], [np.nan, 1, 2, 3, 4, 5],
             [1.0, 2.0 ** -53, 2.0 ** -53, 0, 0, 0], [2.0 ** 1000] * 6, [1e-310, -3e-310, 0, 0, 0, 1e-300]]


def _same_bits(got, want):
    return (got.view(np.uint64) == want.view(np.uint64)) | (np.isnan(got) & np.isnan(want))


def test_host_build_matches_model():
    """The C++ of the kernel's sum, compiled for the host (the library's
    bbpp_neighbour_sums_host), bit for bit against the model."""
    import bbpp
    try:
        bbpp.lib()
    except OSError as e:
        pytest.skip(str(e))
    v = sample(20000, 4)
    v[:len(EDGE_ROWS)] = EDGE_ROWS
    got = bbpp.neighbour_sums(v, host=True)
    want = np.array([model(row)[0] for row in v])
    same = _same_bits(got, want)
    assert same.all(), np.flatnonzero(~same)[:10]


@pytest.mark.gpu
def test_gpu_neighbour_sums_match_model():
    import bbpp
    v = sample(20000, 3)
    v[:len(EDGE_ROWS)] = EDGE_ROWS
    got = bbpp.neighbour_sums(v)
    want = np.array([model(row)[0] for row in v])
    same = _same_bits(got, want)
    assert same.all(), np.flatnonzero(~same)[:10]
    assert _same_bits(got, bbpp.neighbour_sums(v, host=True)).all()


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["fp64", "fp32_ir"])
def test_gpu_solve_with_and_without_exact_sums(method):
    """Solves with the integer neighbour sums and with FP64 adds (the plain
    FP64 method's search kernel; the FP64 residuals of the mixed method): same
    iteration count within 2, solutions within 1e-12 of each other (relative,
    max norm; the mixed method's FP32 inner iterations, 1e-9), both to
    tolerance."""
    import bbpp
    from bbpp import problems
    g = problems.make_grid(96, "ppn")
    cents, radii = problems.place_spheres(g, 40, 6, 7)
    s = bbpp.Solver(g)
    dmask = bbpp.DeviceArray(g.shape, np.uint8)
    s.sphere_mask(cents, radii, dmask)
    seq = problems.OUSequence(g.shape, 7, dmask.download())
    seq.field()
    rhs = seq.step()
    drhs = bbpp.DeviceArray.from_host(rhs)
    prec, tol, close = (bbpp.FP64, 1e-11, 1e-12) if method == "fp64" else (bbpp.FP32_IR, 1e-10, 1e-9)
    out = {}
    for on in (True, False):
        s.set_xsum(on)
        dx = bbpp.DeviceArray(g.shape, np.float64)
        r = s.solve(drhs, dx, dmask, tol=tol, precision=prec)
        assert r.status == 0 and r.true_rel < 1.2 * tol
        out[on] = (r.iters, dx.download())
    assert abs(out[True][0] - out[False][0]) <= 2
    a, b = out[True][1], out[False][1]
    assert np.abs(a - b).max() <= close * np.abs(b).max()
    s.close()
