"""Bluebottle restart files (restart.config-<rank>): the fields of the
pressure solve and its epilogue, read and written in the reference's layout.

The reference writes a restart as raw native-endian arrays in this order
(out_restart, src/domain.c:3005-3090; read back by in_restart, :3093-3200):

    ttime dt0 dt (real) stepnum rec_vtk_stepnum_out (int)
    rec_cgns_flow_ttime_out rec_cgns_part_ttime_out rec_vtk_ttime_out (real)
    u u0 diff0_u conv0_u diff_u conv_u u_star      (real, Gfx.s3b each)
    v v0 diff0_v conv0_v diff_v conv_v v_star      (real, Gfy.s3b each)
    w w0 diff0_w conv0_w diff_w conv_w w_star      (real, Gfz.s3b each)
    p phi p0 (real, Gcc.s3b) phase phase_shell (int, Gcc.s3b)
    flag_u flag_v flag_w (int, face s3b)
    nparts_subdom, the particle records, and further scalars (kept as bytes)

with `real` = double (-DDOUBLE).  One rank owns the whole domain here, so
the ghosted sizes are those of the full grid.  `State.solver_inputs()` turns a
restart into what the solver takes: dense u*, v*, w* faces and the solid mask
(phase > -1); `Solver.rhs_div` then builds the right-hand side on the GPU.
"""
import numpy as np

HEADER = (("ttime", "<f8"), ("dt0", "<f8"), ("dt", "<f8"), ("stepnum", "<i4"), ("rec_vtk_stepnum_out", "<i4"),
          ("rec_cgns_flow_ttime_out", "<f8"), ("rec_cgns_part_ttime_out", "<f8"), ("rec_vtk_ttime_out", "<f8"))
FACE_SET = ("{c}", "{c}0", "diff0_{c}", "conv0_{c}", "diff_{c}", "conv_{c}", "{c}_star")
CELL_REAL = ("p", "phi", "p0")
CELL_INT = ("phase", "phase_shell")
FLAGS = ("flag_u", "flag_v", "flag_w")


def sizes(nx, ny, nz):
    """Ghosted sizes (Gcc, Gfx, Gfy, Gfz s3b) of one rank owning nx x ny x nz cells."""
    return ((nx + 2) * (ny + 2) * (nz + 2), (nx + 3) * (ny + 2) * (nz + 2), (nx + 2) * (ny + 3) * (nz + 2),
            (nx + 2) * (ny + 2) * (nz + 3))


def fields(nx, ny, nz):
    """(name, dtype, count) of the array section, in file order."""
    gcc, gfx, gfy, gfz = sizes(nx, ny, nz)
    out = []
    for c, n in (("u", gfx), ("v", gfy), ("w", gfz)):
        out += [(f.format(c=c), "<f8", n) for f in FACE_SET]
    out += [(f, "<f8", gcc) for f in CELL_REAL]
    out += [(f, "<i4", gcc) for f in CELL_INT]
    out += [("flag_u", "<i4", gfx), ("flag_v", "<i4", gfy), ("flag_w", "<i4", gfz)]
    return out


class State:
    """A restart's header scalars, its arrays (1-D, ghosted, the reference's
    layouts) and the undecoded tail (particles and later records)."""

    def __init__(self, dims, header, arrays, tail=b""):
        self.dims = tuple(int(v) for v in dims)
        self.header = dict(header)
        self.arrays = dict(arrays)
        self.tail = bytes(tail)

    # dense views (x fastest), the layouts of the oracle and of bbpp_rhs_div
    def cells(self, name):
        nx, ny, nz = self.dims
        return self.arrays[name].reshape(nz + 2, ny + 2, nx + 2)[1:-1, 1:-1, 1:-1].copy()

    def faces(self, c):
        """Dense u*, v* or w* (c = 'u', 'v', 'w') of the interior faces."""
        nx, ny, nz = self.dims
        a = self.arrays[c + "_star"]
        if c == "u":  # GFX_LOC = j + k s1b + i s2b
            return a.reshape(nx + 3, nz + 2, ny + 2)[1:-1, 1:-1, 1:-1].transpose(1, 2, 0).copy()
        if c == "v":  # GFY_LOC = k + i s1b + j s2b
            return a.reshape(ny + 3, nx + 2, nz + 2)[1:-1, 1:-1, 1:-1].transpose(2, 0, 1).copy()
        return a.reshape(nz + 3, ny + 2, nx + 2)[1:-1, 1:-1, 1:-1].copy()  # GFZ_LOC = i + j s1b + k s2b

    def mask(self):
        """Solid cells of the interior: phase > -1 (src/cuda_solver.cu, part_BC_p)."""
        return (self.cells("phase") > -1).astype(np.uint8)

    def solver_inputs(self):
        """(u*, v*, w* dense faces, mask, dt) for Solver.rhs_div and Solver.solve."""
        return self.faces("u"), self.faces("v"), self.faces("w"), self.mask(), float(self.header["dt"])


def read(path, dims):
    """Read a one-rank restart of an nx x ny x nz grid."""
    nx, ny, nz = dims
    raw = open(path, "rb").read()
    off = 0
    header = {}
    for name, dt in HEADER:
        v = np.frombuffer(raw, dtype=dt, count=1, offset=off)[0]
        header[name] = v.item()
        off += np.dtype(dt).itemsize
    arrays = {}
    for name, dt, n in fields(nx, ny, nz):
        nbytes = n * np.dtype(dt).itemsize
        if off + nbytes > len(raw):
            raise ValueError("restart file %s is shorter than a %dx%dx%d grid needs" % (path, nx, ny, nz))
        arrays[name] = np.frombuffer(raw, dtype=dt, count=n, offset=off).copy()
        off += nbytes
    return State(dims, header, arrays, raw[off:])


def write(path, state):
    """Write a restart in the reference's order; arrays missing from the state
    are written as zeros, and an empty tail as no particles (nparts_subdom = 0,
    ncoeffs_max = 0, pid_int = pid_back = gradP.z = 0)."""
    nx, ny, nz = state.dims
    with open(path, "wb") as f:
        for name, dt in HEADER:
            np.array([state.header.get(name, 0)], dtype=dt).tofile(f)
        for name, dt, n in fields(nx, ny, nz):
            a = state.arrays.get(name)
            a = np.zeros(n, dt) if a is None else np.ascontiguousarray(a, dtype=dt).ravel()
            if a.size != n:
                raise ValueError("%s has %d values, the layout needs %d" % (name, a.size, n))
            a.tofile(f)
        if state.tail:
            f.write(state.tail)
        else:
            np.array([0, 0], "<i4").tofile(f)          # nparts_subdom, ncoeffs_max
            np.zeros(3, "<f8").tofile(f)               # pid_int, pid_back, gradP.z
