"""The z chunking of the stencil kernels (bbpp_z_chunks in
bluebottle-3.0_gb300/csrc/bbpp_internal.h, exported as bbpp_plan_z_chunks):
host arithmetic, checked on the CPU against a restatement and against the
launch shapes measured at 256^3 and 512^3."""
import os
import sys

import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "bluebottle-3.0_gb300"))
import bbpp  # noqa: E402


def restated(units, nz, slots, min_kz):
    def norm(c):
        k = -(-nz // c)
        if k < min_kz and nz >= min_kz:
            k = min_kz
        return -(-nz // k), k

    best, kz = norm(max(1, min(slots // units, nz)))
    if units * best >= 0.9 * slots:
        return best, kz
    tbest = None
    for c in range(1, nz + 1):
        cc, k = norm(c)
        if cc != c:
            continue
        t = -(-(units * cc) // slots) * (k + 2)
        if tbest is None or t < tbest:
            tbest, best, kz = t, cc, k
    return best, kz


@pytest.fixture(scope="module")
def lib_ok():
    try:
        bbpp.lib()
    except OSError as e:
        pytest.skip(str(e))


def test_measured_shapes(lib_ok):
    # 256^3: FP64 search (4 x 16 tiles of 64 x 16), fused kernel (64 slabs), 3 CTAs on 152 SMs
    assert bbpp.plan_z_chunks(64, 256, 456, 8) == (7, 37)
    assert bbpp.plan_z_chunks(64, 256, 456, 1) == (7, 37)
    # 512^3: 256 tile columns against 456 slots (one wave only 56% full) -> 7 chunks in 4 waves
    assert bbpp.plan_z_chunks(256, 512, 456, 8) == (7, 74)
    # 512^3 fused kernel on 2-row slabs: 256 slabs, 2 CTAs per SM
    assert bbpp.plan_z_chunks(256, 512, 304, 1) == (7, 74)


def test_matches_restatement_and_covers_every_plane(lib_ok):
    for units in (1, 7, 64, 100, 128, 256, 1000, 5000):
        for nz in (1, 3, 8, 17, 64, 100, 256, 512):
            for slots in (152, 304, 456, 608):
                for min_kz in (1, 4, 8):
                    got = bbpp.plan_z_chunks(units, nz, slots, min_kz)
                    assert got == restated(units, nz, slots, min_kz), (units, nz, slots, min_kz)
                    n, kz = got
                    assert 1 <= n <= nz and n * kz >= nz and (n - 1) * kz < nz
                    if nz >= min_kz:
                        assert kz >= min_kz


def test_full_waves_kept(lib_ok):
    """Where one wave fills at least 90% of the slots the count is slots // units."""
    for units, slots in ((64, 456), (50, 152), (150, 152)):
        n, _ = bbpp.plan_z_chunks(units, 4096, slots, 1)
        assert n == slots // units


def test_bad_arguments(lib_ok):
    for args in ((0, 8, 152, 1), (8, 0, 152, 1), (8, 8, 0, 1), (8, 8, 152, 0)):
        with pytest.raises(bbpp.BbppError):
            bbpp.plan_z_chunks(*args)
