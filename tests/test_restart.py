"""Bluebottle restart files (src/domain.c:3005-3200) and the right-hand side
they feed: round trips through bbpp.restart, the layouts against the ghosted
layouts of the drop-in tests, and the GPU rhs builder against the reference's
PP_rhs fixture."""
import os
import sys

import numpy as np
import pytest

from bbpp import restart

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import layout  # noqa: E402

from test_golden import load  # noqa: E402


def random_state(dims, seed, with_tail=False):
    rng = np.random.default_rng(seed)
    arrays = {}
    for name, dt, n in restart.fields(*dims):
        arrays[name] = rng.normal(size=n) if dt == "<f8" else rng.integers(-1, 3, n).astype(np.int32)
    header = {"ttime": 1.5, "dt0": 1e-3, "dt": 2e-3, "stepnum": 17, "rec_vtk_stepnum_out": 3,
              "rec_cgns_flow_ttime_out": 0.25, "rec_cgns_part_ttime_out": 0.5, "rec_vtk_ttime_out": 0.75}
    tail = rng.bytes(123) if with_tail else b""
    return restart.State(dims, header, arrays, tail)


@pytest.mark.parametrize("with_tail", [False, True])
def test_round_trip(tmp_path, with_tail):
    dims = (6, 5, 4)
    st = random_state(dims, 3, with_tail)
    path = str(tmp_path / "restart.config-0")
    restart.write(path, st)
    gcc, gfx, gfy, gfz = restart.sizes(*dims)
    arrays = 8 * (7 * (gfx + gfy + gfz) + 3 * gcc) + 4 * (2 * gcc + gfx + gfy + gfz)
    tail = len(st.tail) if with_tail else 8 + 24
    assert os.path.getsize(path) == 56 + arrays + tail
    back = restart.read(path, dims)
    assert back.header == st.header
    for name in st.arrays:
        assert np.array_equal(back.arrays[name], st.arrays[name])
    if with_tail:
        assert back.tail == st.tail


def test_short_file_rejected(tmp_path):
    path = str(tmp_path / "r")
    restart.write(path, random_state((4, 4, 4), 1))
    with pytest.raises(ValueError):
        restart.read(path, (5, 4, 4))


def test_dense_views_match_reference_layouts():
    dims = (7, 5, 3)
    nx, ny, nz = dims
    rng = np.random.default_rng(9)
    u, v, w = rng.normal(size=(nz, ny, nx + 1)), rng.normal(size=(nz, ny + 1, nx)), rng.normal(size=(nz + 1, ny, nx))
    ph = np.where(rng.random((nz, ny, nx)) < 0.2, 0, -1)
    st = random_state(dims, 2)
    st.arrays["u_star"], st.arrays["v_star"], st.arrays["w_star"] = (layout.fx_to_s3b(u), layout.fy_to_s3b(v),
                                                                    layout.fz_to_s3b(w))
    st.arrays["phase"] = layout.cells_to_s3b(ph.astype(float)).astype(np.int32)
    fu, fv, fw, mask, dt = st.solver_inputs()
    assert np.array_equal(fu, u) and np.array_equal(fv, v) and np.array_equal(fw, w)
    assert np.array_equal(mask, (ph > -1).astype(np.uint8)) and dt == 2e-3


def test_restart_rhs_matches_reference_fixture(orc, tmp_path):
    """The reference's PP_rhs fixture, reproduced from faces that went through
    a restart file (oracle arithmetic, bit for bit)."""
    d = load("rhs_ppn")
    dims = d["dims"]
    st = random_state(dims, 5)
    st.arrays["u_star"], st.arrays["v_star"], st.arrays["w_star"] = (layout.fx_to_s3b(d["u"]),
                                                                    layout.fy_to_s3b(d["v"]),
                                                                    layout.fz_to_s3b(d["w"]))
    st.header["dt"] = float(d["dt"])
    path = str(tmp_path / "restart.config-0")
    restart.write(path, st)
    fu, fv, fw, mask, dt = restart.read(path, dims).solver_inputs()
    g = orc.grid(*dims, *d["h"], bc=d["bc"])
    assert np.array_equal(orc.rhs_div(g, float(d["rho_f"]), dt, fu, fv, fw), d["rhs"])


@pytest.mark.gpu
def test_gpu_rhs_div_matches_reference_fixture(bbpp_lib):
    import bbpp
    d = load("rhs_ppn")
    g = bbpp.Grid.make(*d["dims"], *d["h"], bc=d["bc"])
    s = bbpp.Solver(g)
    du, dv, dw = (bbpp.DeviceArray.from_host(np.ascontiguousarray(d[k])) for k in ("u", "v", "w"))
    out = bbpp.DeviceArray(g.shape, np.float64)
    s.rhs_div(float(d["rho_f"]), float(d["dt"]), du, dv, dw, out)
    assert np.array_equal(out.download(), d["rhs"])
