"""The drop-in entry points (include/bbpp_bluebottle.h) called the way the
Bluebottle time loop calls them (src/bluebottle.c:139,228-234), with a stub
host program that owns the reference's globals (tests/dropin/host_stub.c).

Checked against whole reference solves (golden dropin_*.npz: PP_rhs from
u*, v*, w*, particle masking, coeffs_refine, cuda_PP_cg[_noparts]) and the
oracle.
"""
import ctypes
import json
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
BUILD = os.path.join(ROOT, "tests", "_build")
MANIFEST = json.load(open(os.path.join(GOLD, "manifest.json")))
DROPIN = sorted(k for k, v in MANIFEST.items() if v["kind"] == "dropin")


class GridInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "is_ ie in_ isb ieb inb js je jn jsb jeb jnb ks ke kn ksb keb knb "
        "_is _ie _isb _ieb _js _je _jsb _jeb _ks _ke _ksb _keb "
        "s1 s1b s2 s2b s3 s3b s2_i s2_j s2_k s2b_i s2b_j s2b_k").split()]


D, I = ctypes.c_double, ctypes.c_int


class DomStruct(ctypes.Structure):
    _fields_ = [("Gcc", GridInfo), ("Gfx", GridInfo), ("Gfy", GridInfo), ("Gfz", GridInfo),
                ("xs", D), ("xe", D), ("xl", D), ("xn", I), ("dx", D),
                ("ys", D), ("ye", D), ("yl", D), ("yn", I), ("dy", D),
                ("zs", D), ("ze", D), ("zl", D), ("zn", I), ("dz", D),
                ("rank", I), ("e", I), ("w", I), ("n", I), ("s", I), ("t", I), ("b", I),
                ("I", I), ("Is", I), ("Ie", I), ("In", I), ("J", I), ("Js", I), ("Je", I), ("Jn", I),
                ("K", I), ("Ks", I), ("Ke", I), ("Kn", I), ("S1", I), ("S2", I), ("S3", I)]


def fill(g, n):
    """grid_info of one rank, as domain_fill (src/domain.c:918-1487)."""
    (ni, nj, nk) = n
    for ax, m in zip("ijk", n):
        setattr(g, ax + "s" if ax != "i" else "is_", 1)
        setattr(g, ax + "sb", 0)
        setattr(g, ax + "n" if ax != "i" else "in_", m)
        setattr(g, ax + "nb", m + 2)
        setattr(g, ax + "e", m)
        setattr(g, ax + "eb", m + 1)
        setattr(g, "_" + ax + "s", 1)
        setattr(g, "_" + ax + "sb", 0)
        setattr(g, "_" + ax + "e", m)
        setattr(g, "_" + ax + "eb", m + 1)


def make_dom(nx, ny, nz, h):
    d = DomStruct()
    fill(d.Gcc, (nx, ny, nz))
    g = d.Gcc
    g.s1, g.s2, g.s3 = nx, nx * ny, nx * ny * nz
    g.s1b, g.s2b, g.s3b = nx + 2, (nx + 2) * (ny + 2), (nx + 2) * (ny + 2) * (nz + 2)
    fill(d.Gfx, (nx + 1, ny, nz))
    f = d.Gfx  # GFX_LOC = j + k s1b + i s2b
    f.s1, f.s2 = ny, ny * nz
    f.s3 = f.s2 * (nx + 1)
    f.s1b, f.s2b = ny + 2, (ny + 2) * (nz + 2)
    f.s3b = f.s2b * (nx + 3)
    fill(d.Gfy, (nx, ny + 1, nz))
    f = d.Gfy  # GFY_LOC = k + i s1b + j s2b
    f.s1, f.s2 = nz, nz * nx
    f.s3 = f.s2 * (ny + 1)
    f.s1b, f.s2b = nz + 2, (nz + 2) * (nx + 2)
    f.s3b = f.s2b * (ny + 3)
    fill(d.Gfz, (nx, ny, nz + 1))
    f = d.Gfz  # GFZ_LOC = i + j s1b + k s2b
    f.s1, f.s2 = nx, nx * ny
    f.s3 = f.s2 * (nz + 1)
    f.s1b, f.s2b = nx + 2, (nx + 2) * (ny + 2)
    f.s3b = f.s2b * (nz + 3)
    d.xn, d.yn, d.zn = nx, ny, nz
    d.dx, d.dy, d.dz = h
    d.xl, d.yl, d.zl = nx * h[0], ny * h[1], nz * h[2]
    d.xe, d.ye, d.ze = d.xl, d.yl, d.zl
    d.In = d.Jn = d.Kn = d.S1 = d.S2 = d.S3 = 1
    return d


def faces_to_ref(u, v, w):
    """Dense face arrays -> the reference's ghosted, permuted face layouts."""
    nz, ny, nx1 = u.shape
    nx = nx1 - 1
    U = np.zeros((nx + 3, nz + 2, ny + 2))       # [I, K, J]
    U[1:nx + 2, 1:nz + 1, 1:ny + 1] = u.transpose(2, 0, 1)
    V = np.zeros((ny + 3, nx + 2, nz + 2))       # [J, I, K]
    V[1:ny + 2, 1:nx + 1, 1:nz + 1] = v.transpose(1, 2, 0)
    W = np.zeros((nz + 3, ny + 2, nx + 2))       # [K, J, I]
    W[1:nz + 2, 1:ny + 1, 1:nx + 1] = w
    return U, V, W


def phase_b(mask, bc):
    nz, ny, nx = mask.shape
    ph = -np.ones((nz + 2, ny + 2, nx + 2), np.int32)
    ph[1:-1, 1:-1, 1:-1] = np.where(mask > 0, 0, -1)
    if bc[0] == 0:
        ph[:, :, 0], ph[:, :, -1] = ph[:, :, -2], ph[:, :, 1]
    if bc[2] == 0:
        ph[:, 0, :], ph[:, -1, :] = ph[:, -2, :], ph[:, 1, :]
    if bc[4] == 0:
        ph[0], ph[-1] = ph[-2], ph[1]
    return ph


def flags_b(mask, bc, dims):
    """Face flags in the reference's ghosted face layouts, by the rule the
    host pin builds them with (cage_flag_*: -1 on a fluid/solid face;
    flag_external_*: 0 on the wall faces of a non-periodic direction; else 1)."""
    nx, ny, nz = dims
    ph = phase_b(mask if mask is not None else np.zeros((nz, ny, nx), np.uint8), bc)
    fl = ph < 0
    U = np.ones((nx + 3, nz + 2, ny + 2), np.int32)   # [I, K, J]
    U[1:nx + 2] = np.where(fl[:, :, :-1] != fl[:, :, 1:], -1, 1).transpose(2, 0, 1)
    if bc[0] != 0:
        U[1], U[nx + 1] = 0, 0
    V = np.ones((ny + 3, nx + 2, nz + 2), np.int32)   # [J, I, K]
    V[1:ny + 2] = np.where(fl[:, :-1, :] != fl[:, 1:, :], -1, 1).transpose(1, 2, 0)
    if bc[2] != 0:
        V[1], V[ny + 1] = 0, 0
    W = np.ones((nz + 3, ny + 2, nx + 2), np.int32)   # [K, J, I]
    W[1:nz + 2] = np.where(fl[:-1] != fl[1:], -1, 1)
    if bc[4] != 0:
        W[1], W[nz + 1] = 0, 0
    return U, V, W


def load(name):
    d = dict(np.load(os.path.join(GOLD, name + ".npz")))
    d["dims"] = tuple(int(x) for x in d["dims"])
    d["bc"] = tuple(int(x) for x in d["bc"])
    d["h"] = tuple(float(x) for x in d["h"])
    d["mask"] = None if d["mask"].size == 0 else d["mask"]
    return d


def faces_dense_check(d):
    nx, ny, nz = d["dims"]
    assert d["u"].shape == (nz, ny, nx + 1) and d["w"].shape == (nz + 1, ny, nx)


# ------------------------------------------------------------------ CPU ---
@pytest.mark.parametrize("name", DROPIN)
def test_oracle_whole_solve_matches_reference(orc, name):
    d = load(name)
    faces_dense_check(d)
    g = orc.grid(*d["dims"], *d["h"], bc=d["bc"])
    rhs = orc.rhs_div(g, float(d["rho_f"]), float(d["dt"]), d["u"], d["v"], d["w"])
    if d["mask"] is not None:
        rhs = orc.rhs_mask_refine(g, d["mask"], rhs)
    x, res = orc.pcg(g, rhs, d["mask"], tol=float(d["pp_residual"]), stop=0)
    assert res["iters"] == int(d["niter"])
    assert np.linalg.norm(x - d["phi"]) <= 1e-12 * np.linalg.norm(d["phi"])


def test_dropin_exports():
    import bbpp
    if not os.path.exists(bbpp.DROPIN_LIBPATH):
        pytest.skip("drop-in library not built")
    out = subprocess.run(["nm", "-D", "--defined-only", bbpp.DROPIN_LIBPATH], capture_output=True, text=True,
                         check=True).stdout
    syms = {l.split()[-1] for l in out.splitlines() if l.strip()}
    for s in ("cuda_PP_init_jacobi_preconditioner", "cuda_PP_cg", "cuda_PP_cg_noparts", "cuda_PP_cg_timed",
              "cuda_dom_BC_p", "cuda_project", "cuda_update_p", "cuda_build_cages", "bbpp_bluebottle_release"):
        assert s in syms
    und = subprocess.run(["nm", "-D", "-u", bbpp.DROPIN_LIBPATH], capture_output=True, text=True,
                         check=True).stdout
    for s in ("dom", "_phi", "_rhs_p", "_u_star", "_phase", "pp_residual", "recorder_PP", "cuda_part_BC_p"):
        assert s in und  # resolved from the host program at load time


# ------------------------------------------------------------------ GPU ---
def build_stub():
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "libbbhost.so")
    src = os.path.join(ROOT, "tests", "dropin", "host_stub.c")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        subprocess.run(["gcc", "-shared", "-fPIC", "-O2", "-DBBPP_BLUEBOTTLE_IMPL", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(cuda, "include"), src, "-o", out, "-L", os.path.join(cuda, "lib64"),
                        "-lcudart"], check=True)
    return out


class Host:
    """The stub host program plus the drop-in library, loaded globally."""

    def __init__(self):
        import bbpp
        self.bbpp = bbpp
        self.stub = ctypes.CDLL(build_stub(), mode=ctypes.RTLD_GLOBAL)
        ctypes.CDLL(bbpp.LIBPATH, mode=ctypes.RTLD_GLOBAL)
        self.lib = ctypes.CDLL(bbpp.DROPIN_LIBPATH, mode=ctypes.RTLD_GLOBAL)
        self.keep = []

    def g(self, name, ctype):
        return ctype.in_dll(self.stub, name)

    def dev(self, arr):
        d = self.bbpp.DeviceArray.from_host(np.ascontiguousarray(arr))
        self.keep.append(d)
        return d.ptr

    def setup(self, d, pp_residual, pp_max_iter=20000):
        nx, ny, nz = d["dims"]
        self.dom = make_dom(nx, ny, nz, d["h"])
        self.g("dom", ctypes.c_void_p).value = ctypes.addressof(self.dom)
        bc = (ctypes.c_int * 6).in_dll(self.stub, "bc")
        for i, b in enumerate(d["bc"]):
            bc[i] = b
        self.g("rank", ctypes.c_int).value = 0
        self.g("nprocs", ctypes.c_int).value = 1
        parts = d["mask"] is not None
        self.g("NPARTS", ctypes.c_int).value = 1 if parts else 0
        self.g("nparts", ctypes.c_int).value = 1 if parts else 0
        self.g("rho_f", ctypes.c_double).value = float(d["rho_f"])
        self.g("dt", ctypes.c_double).value = float(d["dt"])
        self.g("pp_residual", ctypes.c_double).value = pp_residual
        self.g("pp_max_iter", ctypes.c_int).value = pp_max_iter
        U, V, W = faces_to_ref(d["u"], d["v"], d["w"])
        for nm, a in (("_u_star", U), ("_v_star", V), ("_w_star", W)):
            self.g(nm, ctypes.c_void_p).value = self.dev(a)
        n3b = (nx + 2) * (ny + 2) * (nz + 2)
        self.g("_phi", ctypes.c_void_p).value = self.dev(np.full(n3b, 7.0))
        self.g("_rhs_p", ctypes.c_void_p).value = self.dev(np.zeros(n3b))
        self.g("_invM", ctypes.c_void_p).value = self.dev(np.zeros(nx * ny * nz))
        if parts:
            ph = phase_b(d["mask"], d["bc"])
            self.phase_host = np.ascontiguousarray(ph.ravel())
            self.g("_phase", ctypes.c_void_p).value = self.dev(self.phase_host)
            self.stub.stub_set_phase_host(self.phase_host.ctypes.data, ctypes.c_longlong(n3b))

    def phi(self, d):
        nx, ny, nz = d["dims"]
        ptr = self.g("_phi", ctypes.c_void_p).value
        out = np.empty((nz + 2) * (ny + 2) * (nx + 2))
        self.bbpp.lib().bbpp_d2h(out.ctypes.data, ptr, out.nbytes)
        return out.reshape(nz + 2, ny + 2, nx + 2)


@pytest.mark.gpu
@pytest.mark.parametrize("name", DROPIN)
def test_dropin_matches_reference(bbpp_lib, orc, name):
    d = load(name)
    H = Host()
    H.setup(d, float(d["pp_residual"]))
    H.lib.cuda_PP_init_jacobi_preconditioner()
    if d["mask"] is not None:
        H.lib.cuda_PP_cg()
    else:
        H.lib.cuda_PP_cg_noparts()
    phi = H.phi(d)
    inner = phi[1:-1, 1:-1, 1:-1]
    assert np.linalg.norm(inner - d["phi"]) <= 1e-10 * np.linalg.norm(d["phi"])
    assert (phi[0] == 7.0).all()  # ghosts are the caller's
    assert abs(H.g("stub_niter", ctypes.c_int).value - int(d["niter"])) <= 1
    assert H.g("stub_name", ctypes.c_char * 256).value == b"solver_expd.rec"
    resid = H.g("stub_resid", ctypes.c_double).value
    assert resid <= float(d["pp_residual"])
    # _invM as PP_jacobi_init
    nx, ny, nz = d["dims"]
    inv = np.empty(nx * ny * nz)
    H.bbpp.lib().bbpp_d2h(inv.ctypes.data, H.g("_invM", ctypes.c_void_p).value, inv.nbytes)
    assert np.array_equal(inv.reshape(nz, ny, nx), orc.invm(orc.grid(*d["dims"], *d["h"], bc=d["bc"])))
    # the timed variant records per-phase device times
    if d["mask"] is not None:
        H.g("_phi", ctypes.c_void_p)
        H.lib.cuda_PP_cg_timed()
        assert H.g("stub_timed_calls", ctypes.c_int).value == 1
        assert H.g("stub_init_timed", ctypes.c_int).value == 1
        assert H.g("stub_spmv", ctypes.c_double).value > 0
        assert np.linalg.norm(H.phi(d)[1:-1, 1:-1, 1:-1] - d["phi"]) <= 1e-10 * np.linalg.norm(d["phi"])
    H.lib.bbpp_bluebottle_release()


@pytest.mark.gpu
def test_dropin_max_iter_exits_like_reference(bbpp_lib):
    """pp_max_iter exceeded: the reference prints and exit(EXIT_FAILURE)s
    (src/cuda_solver.cu:271-279); run in a child process."""
    code = textwrap.dedent("""
        import sys
        sys.path[:0] = %r
        import test_dropin as T
        d = T.load(%r)
        H = T.Host()
        H.setup(d, 1e-14, pp_max_iter=3)
        H.lib.cuda_PP_init_jacobi_preconditioner()
        H.lib.cuda_PP_cg()
        print("returned")
    """) % ([os.path.join(ROOT, "tests"), os.path.join(ROOT, "bluebottle-3.0_gb300"), os.path.join(ROOT, "oracle")],
           [n for n in DROPIN if "spheres" in n][0])
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 1, r.stdout + r.stderr
    assert "did not converge" in r.stdout and "returned" not in r.stdout


# ------------------------------------------------------------ epilogue ----
EPI = sorted(k for k, v in json.load(open(os.path.join(GOLD, "manifest.json"))).items() if v["kind"] == "epilogue")
REFLIB = os.path.join(ROOT, "oracle", "_ref", "libref.so")


@pytest.mark.skipif(not os.path.exists(REFLIB), reason="host build of the reference not present")
@pytest.mark.parametrize("dims,bc,frac", [((7, 6, 5), (0, 0, 0, 0, 2, 2), 0.2), ((6, 8, 4), (2,) * 6, 0.3),
                                          ((5, 4, 6), (0,) * 6, 0.0)])
def test_flags_helper_matches_reference_host(dims, bc, frac):
    """The face flags the drop-in epilogue test gives the library are the
    ones the reference's host pin builds."""
    sys.path.insert(0, GOLD)
    import make_golden
    L = make_golden.load()
    L.ref_flags.argtypes = [ctypes.c_void_p] * 4
    nx, ny, nz = dims
    rng = np.random.default_rng(nx * ny)
    mask = (rng.random((nz, ny, nx)) < frac).astype(np.uint8) if frac else None
    make_golden.setup(L, dims, (1 / nx, 1 / ny, 1 / nz), bc, mask)
    U, V, W = flags_b(mask, bc, dims)
    fu, fv, fw = (np.zeros(a.size, np.int32) for a in (U, V, W))
    ph = np.zeros((nx + 2) * (ny + 2) * (nz + 2), np.int32)
    L.ref_flags(fu.ctypes.data, fv.ctypes.data, fw.ctypes.data, ph.ctypes.data)
    assert np.array_equal(fu, U.ravel()) and np.array_equal(fv, V.ravel()) and np.array_equal(fw, W.ravel())
    m = mask if mask is not None else np.zeros((nz, ny, nx), np.uint8)
    assert np.array_equal(ph, phase_b(m, bc).ravel())


def periodic_ghosts(a, bc):
    """The host's one-rank mpi_cuda_exchange_Gcc on a (nz+2, ny+2, nx+2) array."""
    a = a.copy()
    if bc[0] == 0:
        a[:, :, 0], a[:, :, -1] = a[:, :, -2], a[:, :, 1]
    if bc[2] == 0:
        a[:, 0, :], a[:, -1, :] = a[:, -2, :], a[:, 1, :]
    if bc[4] == 0:
        a[0], a[-1] = a[-2], a[1]
    return a


@pytest.mark.gpu
@pytest.mark.parametrize("name", EPI)
def test_dropin_epilogue_matches_reference(bbpp_lib, name):
    """cuda_dom_BC_p(_phi), cuda_project(), cuda_update_p() after a solve, on
    the reference's ghosted arrays: ghosts and u, v, w equal the reference's
    kernels bit for bit; p to rounding (the mean is summed in another order)."""
    sys.path.insert(0, GOLD)
    import layout
    d = load(name)
    nx, ny, nz = d["dims"]
    H = Host()
    H.setup(dict(d, u=d["us"], v=d["vs"], w=d["ws"]), 1e-8)
    bc = d["bc"]
    # phi with the host's periodic exchange done, as the time loop has it
    phib = np.zeros((nz + 2, ny + 2, nx + 2))
    phib[1:-1, 1:-1, 1:-1] = d["phi"]
    phib = periodic_ghosts(phib, bc)
    pptr = H.dev(phib.ravel())
    H.g("_phi", ctypes.c_void_p).value = pptr
    H.lib.cuda_dom_BC_p(ctypes.c_void_p(pptr))
    got = np.empty(phib.size)
    H.bbpp.lib().bbpp_sync()
    H.bbpp.lib().bbpp_d2h(got.ctypes.data, pptr, got.nbytes)
    assert np.array_equal(got, d["phi_b"])
    # projection
    U, V, W = flags_b(d["mask"], bc, d["dims"])
    for nm, a in (("_flag_u", U), ("_flag_v", V), ("_flag_w", W)):
        H.g(nm, ctypes.c_void_p).value = H.dev(np.ascontiguousarray(a.ravel()))
    outs = {}
    for nm, size in (("_u", U.size), ("_v", V.size), ("_w", W.size)):
        outs[nm] = H.dev(np.zeros(size))
        H.g(nm, ctypes.c_void_p).value = outs[nm]
    H.lib.cuda_project()
    H.bbpp.lib().bbpp_sync()
    for nm, conv, ref in (("_u", layout.fx_from_s3b, d["u"]), ("_v", layout.fy_from_s3b, d["v"]),
                          ("_w", layout.fz_from_s3b, d["w"])):
        size = {"_u": U.size, "_v": V.size, "_w": W.size}[nm]
        b = np.empty(size)
        H.bbpp.lib().bbpp_d2h(b.ctypes.data, outs[nm], b.nbytes)
        assert np.array_equal(conv(b, d["dims"]), ref)
    # pressure update
    if d["mask"] is None:
        ph = phase_b(np.zeros((nz, ny, nx), np.uint8), bc)
        H.g("_phase", ctypes.c_void_p).value = H.dev(np.ascontiguousarray(ph.ravel()))
    H.g("_p0", ctypes.c_void_p).value = H.dev(layout.cells_to_s3b(d["p0"]))
    pp = H.dev(np.zeros(phib.size))
    H.g("_p", ctypes.c_void_p).value = pp
    H.lib.cuda_update_p()
    H.bbpp.lib().bbpp_sync()
    b = np.empty(phib.size)
    H.bbpp.lib().bbpp_d2h(b.ctypes.data, pp, b.nbytes)
    p = layout.cells_from_s3b(b, d["dims"])
    assert np.abs(p - d["p"]).max() <= 1e-14 * np.abs(d["p"]).max()


# ---------------------------------------------------------- cage builder --
CAGES = sorted(k for k, v in MANIFEST.items() if v["kind"] == "cages")


def test_part_struct_stride_matches_reference():
    """BB_PART_STRUCT_BYTES (the stride the cage builder reads _parts with)
    equals sizeof(part_struct) of the reference's own header, as the host build
    of the reference measured it when the cage fixtures were written."""
    import re
    hdr = open(os.path.join(ROOT, "include", "bbpp_bluebottle.h")).read()
    stride = int(re.search(r"#define BB_PART_STRUCT_BYTES (\d+)", hdr).group(1))
    assert CAGES and all(MANIFEST[c]["part_struct_bytes"] == stride for c in CAGES)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CAGES)
def test_dropin_build_cages_matches_reference(bbpp_lib, name):
    """cuda_build_cages through the drop-in library, with the host stub's
    globals, against the reference's cage kernels (golden cages_*.npz):
    phase, phase_shell and the three face-flag arrays, element for element."""
    import re
    d = dict(np.load(os.path.join(GOLD, name + ".npz")))
    nx, ny, nz = (int(v) for v in d["dims"])
    H = Host()
    H.dom = make_dom(nx, ny, nz, tuple(float(v) for v in d["h"]))
    H.g("dom", ctypes.c_void_p).value = ctypes.addressof(H.dom)
    bcs = (ctypes.c_int * 6).in_dll(H.stub, "bc")
    for i, b in enumerate(d["bc"]):
        bcs[i] = int(b)
    H.g("rank", ctypes.c_int).value = 0
    H.g("nprocs", ctypes.c_int).value = 1
    parts = d["parts"].reshape(-1, 4)
    with_parts = int(d["with_parts"])
    H.g("NPARTS", ctypes.c_int).value = with_parts
    H.g("nparts", ctypes.c_int).value = len(parts)
    hdr = open(os.path.join(ROOT, "include", "bbpp_bluebottle.h")).read()
    stride = int(re.search(r"#define BB_PART_STRUCT_BYTES (\d+)", hdr).group(1))
    raw = np.zeros((max(len(parts), 1), stride), np.uint8)
    for n, (x, y, z, r) in enumerate(parts):
        raw[n, 0:4] = np.frombuffer(np.int32(n).tobytes(), np.uint8)
        raw[n, 8:40] = np.frombuffer(np.array([r, x, y, z], np.float64).tobytes(), np.uint8)
    H.g("_parts", ctypes.c_void_p).value = H.dev(raw)
    # outputs start as garbage, except phase and phase_shell without particles,
    # which the reference leaves as they were
    keep = with_parts == 0
    ph0 = d["phase"] if keep else np.full(d["phase"].shape, 7, np.int32)
    sh0 = d["phase_shell"] if keep else np.full(d["phase_shell"].shape, 7, np.int32)
    for nm, a in (("_phase", ph0), ("_phase_shell", sh0), ("_flag_u", np.full(d["flag_u"].shape, 7, np.int32)),
                  ("_flag_v", np.full(d["flag_v"].shape, 7, np.int32)),
                  ("_flag_w", np.full(d["flag_w"].shape, 7, np.int32))):
        H.g(nm, ctypes.c_void_p).value = H.dev(np.ascontiguousarray(a, np.int32))
    H.lib.cuda_build_cages()
    H.bbpp.sync()
    for nm, k in (("_phase", "phase"), ("_phase_shell", "phase_shell"), ("_flag_u", "flag_u"), ("_flag_v", "flag_v"),
                  ("_flag_w", "flag_w")):
        out = np.empty(d[k].shape, np.int32)
        H.bbpp.lib().bbpp_d2h(out.ctypes.data, H.g(nm, ctypes.c_void_p).value, out.nbytes)
        assert np.array_equal(out, d[k]), k
