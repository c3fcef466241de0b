"""The oracle-side input generator (oracle/pyproblems.py) against the solver
package's (bbpp.problems): identical sphere centres, masks and right-hand
sides from the same seeds, so the CPU arm of the benchmark solves exactly the
workload the GPU arm solves without loading the solver's library."""
import numpy as np
import pytest

import pyoracle
import pyproblems


def test_rng_streams_match_library(bbpp_lib):
    import bbpp
    for seed in (1, 3, 12345):
        assert np.array_equal(pyoracle.rng_uniform(seed, 1001, -1.0, 1.0), bbpp.rng_uniform(seed, 1001, -1.0, 1.0))
        assert np.array_equal(pyoracle.rng_gauss(seed, 1001), bbpp.rng_gauss(seed, 1001))


@pytest.mark.parametrize("name", ["C2", "C3", "C4"])
def test_sphere_layout_and_mask_match(bbpp_lib, name):
    from bbpp import problems
    g, solid, cents, radii, seed, tol = pyproblems.workload(name)
    c = problems.CONFIGS[name]
    gg = problems.make_grid(c["n"], c["bc"])
    assert tuple(gg.bc) == tuple(g.bc) and (gg.dx, gg.dy, gg.dz) == (g.dx, g.dy, g.dz)
    pc, pr = problems.place_spheres(gg, c["nsph"], c["rad"], c["seed"])
    assert np.array_equal(cents, pc) and np.array_equal(radii, pr)
    assert np.array_equal(solid, problems.sphere_mask_host(gg, pc, pr))
    assert tol == c["tol"] and seed == c["seed"]


def test_ou_sequence_matches(bbpp_lib):
    from bbpp import problems
    g, solid, *_ = pyproblems.workload("C4")
    mine = pyproblems.OUFields((g.nz, g.ny, g.nx), 4, solid)
    theirs = problems.OUSequence((g.nz, g.ny, g.nx), 4, solid)
    assert np.array_equal(mine.current(), theirs.field())
    for _ in range(2):
        assert np.array_equal(mine.advance(), theirs.step())
