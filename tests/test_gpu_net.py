"""GPU checks of the learned initial guess.

Kernel level: the BF16 tensor-core 3x3x3 convolutions (forward on the
mma.sync and tcgen05 kernels, input gradient through the flipped weights,
weight gradient) against torch's FP32 conv3d on
the same BF16 values, with periodic and zero padding and partial tiles.
Network level: loss and gradient of the whole encoder-decoder against the
FP32 CPU reference (oracle/net_oracle.py); training on the GPU lowers the
loss; and the trained guess shortens the PCG compared with the method
without it (zero guess) on held-out right-hand sides.
"""
import numpy as np
import pytest

import bbpp
from bbpp import learned, problems

torch = pytest.importorskip("torch")
import torch.nn.functional as F  # noqa: E402

import net_oracle as NO  # noqa: E402

pytestmark = pytest.mark.gpu


def dev_bf16(a):
    return bbpp.DeviceArray.from_host(NO.bf16_bits(a))


def torch_conv(x, w, px, py, pz):
    """x [N][z][y][x][C] float32 (already BF16 values); w [27][cout][cin]."""
    cout, cin = w.shape[1], w.shape[2]
    xt = torch.as_tensor(x).permute(0, 4, 1, 2, 3)
    wt = torch.as_tensor(w).reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)
    return xt, wt


def conv_ref(xt, wt, px, py, pz):
    x = F.pad(xt, (1, 1, 0, 0, 0, 0), mode="circular" if px else "constant")
    x = F.pad(x, (0, 0, 1, 1, 0, 0), mode="circular" if py else "constant")
    x = F.pad(x, (0, 0, 0, 0, 1, 1), mode="circular" if pz else "constant")
    return F.conv3d(x, wt)


CONVS = [(16, 16), (16, 32), (32, 64), (96, 32), (48, 16)]


@pytest.mark.parametrize("cin,cout", CONVS)
# rows of 128 voxels take a tcgen05 kernel (16 or 32 output channels; 256 too
# for k_conv3_tm, and for k_conv3_tx with 16), the others the mma.sync kernel
@pytest.mark.parametrize("dims,pads", [((20, 12, 6), (1, 1, 0)), ((16, 8, 4), (0, 0, 0)), ((33, 9, 3), (1, 0, 1)),
                                       ((128, 5, 3), (1, 1, 0)), ((256, 2, 5), (0, 1, 1))])
@pytest.mark.parametrize("mode", [1, 2])
def test_conv3_forward_dgrad_wgrad(bbpp_lib, cin, cout, dims, pads, mode):
    L = learned._sig()
    nx, ny, nz = dims
    px, py, pz = pads
    nb = 2
    rng = np.random.default_rng(cin * 7 + cout + nx)
    x = NO.bits_f32(NO.bf16_bits(rng.normal(size=(nb, nz, ny, nx, cin)).astype(np.float32)))
    w = NO.bits_f32(NO.bf16_bits((rng.normal(size=(27, cout, cin)) * 0.1).astype(np.float32)))
    bias = rng.normal(size=cout).astype(np.float32)
    dx, dw = dev_bf16(x), dev_bf16(w)
    db = bbpp.DeviceArray.from_host(bias)
    dy = bbpp.DeviceArray((nb, nz, ny, nx, cout), np.uint16)
    tc0 = L.bbpp_conv3_tc_launches()
    assert L.bbpp_conv3_tc_config(mode, 0) == 0
    try:
        assert L.bbpp_conv3(cin, cout, dx.ptr, cin, 0, dw.ptr, db.ptr, dy.ptr, cout, 0, nx, ny, nz, nb, px, py, pz,
                            0) == 0
    finally:
        L.bbpp_conv3_tc_config(-1, 0)
    # the shapes a tcgen05 kernel takes ran on it
    rows = nx % 128 == 0 if mode == 1 else (nx == 128 or (nx == 256 and cout == 16))
    assert L.bbpp_conv3_tc_launches() - tc0 == (1 if rows and cout in (16, 32) else 0)
    y = NO.bits_f32(dy.download())
    xt, wt = torch_conv(x, w, px, py, pz)
    xt.requires_grad_(True)
    wt.requires_grad_(True)
    yt = conv_ref(xt, wt, px, py, pz)
    yref = (yt + torch.as_tensor(bias).view(1, -1, 1, 1, 1)).detach().permute(0, 2, 3, 4, 1).numpy()
    assert np.abs(y - yref).max() <= 1e-2 * np.abs(yref).max()
    # gradients for an upstream gradient g
    g = NO.bits_f32(NO.bf16_bits(rng.normal(size=(nb, nz, ny, nx, cout)).astype(np.float32)))
    yt.backward(torch.as_tensor(g).permute(0, 4, 1, 2, 3))
    dx_ref = xt.grad.permute(0, 2, 3, 4, 1).numpy()
    dw_ref = wt.grad.permute(2, 3, 4, 0, 1).reshape(27, cout, cin).numpy()
    dg = dev_bf16(g)
    dwt = bbpp.DeviceArray((27, cin, cout), np.uint16)
    assert L.bbpp_conv3_wflip(cin, cout, dw.ptr, dwt.ptr) == 0
    dxin = bbpp.DeviceArray((nb, nz, ny, nx, cin), np.uint16)
    assert L.bbpp_conv3(cout, cin, dg.ptr, cout, 0, dwt.ptr, None, dxin.ptr, cin, 0, nx, ny, nz, nb, px, py, pz,
                        0) == 0
    got_dx = NO.bits_f32(dxin.download())
    assert np.abs(got_dx - dx_ref).max() <= 1e-2 * np.abs(dx_ref).max()
    dW = bbpp.DeviceArray((27, cout, cin), np.float32)
    dW.zero()
    assert L.bbpp_conv3_wgrad(cin, cout, dx.ptr, cin, 0, dg.ptr, cout, dW.ptr, nx, ny, nz, nb, px, py, pz) == 0
    got_dw = dW.download()
    assert np.abs(got_dw - dw_ref).max() <= 2e-4 * np.abs(dw_ref).max()


TC_CONVS = [(16, 16), (16, 32), (96, 32), (48, 16), (32, 16)]


@pytest.mark.parametrize("cin,cout", TC_CONVS)
@pytest.mark.parametrize("dims,pads,nb", [((256, 8, 10), (1, 1, 0), 1), ((128, 6, 12), (1, 1, 0), 2),
                                          ((256, 5, 9), (0, 1, 1), 1)])
@pytest.mark.parametrize("ctas", [1, 5])
@pytest.mark.parametrize("mode", [1, 2])
def test_conv3_tc_marching(bbpp_lib, cin, cout, dims, pads, nb, ctas, mode):
    """The tcgen05 kernels with few CTAs, so each marches through many planes
    and tiles (accumulator ring reuse, segment changes, one- and two-sided
    periodic x wrap), writing into a channel window of a wider output.  Mode 1
    is k_conv3_tm (x-shifted A tiles in tensor memory), mode 2 k_conv3_tx (the
    x-taps stacked in N; rows of 128 voxels, or 256 with 16 output channels)."""
    L = learned._sig()
    nx, ny, nz = dims
    px, py, pz = pads
    rng = np.random.default_rng(cin * 3 + cout + nx + ctas)
    x = NO.bits_f32(NO.bf16_bits(rng.normal(size=(nb, nz, ny, nx, cin)).astype(np.float32)))
    w = NO.bits_f32(NO.bf16_bits((rng.normal(size=(27, cout, cin)) * 0.1).astype(np.float32)))
    bias = rng.normal(size=cout).astype(np.float32)
    dx, dw = dev_bf16(x), dev_bf16(w)
    db = bbpp.DeviceArray.from_host(bias)
    ldo, co_off = cout + 16, 8
    dy = bbpp.DeviceArray((nb, nz, ny, nx, ldo), np.uint16)
    dy.zero()
    tc0 = L.bbpp_conv3_tc_launches()
    assert L.bbpp_conv3_tc_config(mode, ctas) == 0
    try:
        assert L.bbpp_conv3(cin, cout, dx.ptr, cin, 0, dw.ptr, db.ptr, dy.ptr, ldo, co_off, nx, ny, nz, nb, px, py,
                            pz, 1) == 0
    finally:
        L.bbpp_conv3_tc_config(-1, 0)
    taken = mode == 1 or nx == 128 or (nx == 256 and cout == 16)
    assert L.bbpp_conv3_tc_launches() - tc0 == (1 if taken else 0)
    y = NO.bits_f32(dy.download())
    xt, wt = torch_conv(x, w, px, py, pz)
    yref = torch.relu(conv_ref(xt, wt, px, py, pz) + torch.as_tensor(bias).view(1, -1, 1, 1, 1))
    yref = yref.permute(0, 2, 3, 4, 1).numpy()
    assert np.abs(y[..., co_off:co_off + cout] - yref).max() <= 1e-2 * np.abs(yref).max()
    assert not y[..., :co_off].any() and not y[..., co_off + cout:].any()  # channels outside the window untouched


def _small_problem(seed, dims=(16, 16, 8), nb=2):
    nx, ny, nz = dims
    rng = np.random.default_rng(seed)
    rhs = rng.normal(size=(nb, nz, ny, nx)).astype(np.float32)  # residual of the warm start
    prev = rng.normal(size=(nb, nz, ny, nx)).astype(np.float32)
    tgt = (0.01 * rhs + 0.001 * rng.normal(size=(nb, nz, ny, nx))).astype(np.float32)  # correction
    mask = (rng.random((nz, ny, nx)) < 0.05).astype(np.uint8)
    return rhs, prev, tgt, mask


def test_net_gradient_matches_cpu_reference(bbpp_lib):
    net = learned.Net(seed=3)
    p = net.get_params()
    rhs, prev, tgt, mask = _small_problem(1)
    dims = (16, 16, 8)
    d = [bbpp.DeviceArray.from_host(a) for a in (rhs, prev, tgt, mask)]
    h2 = 1.0 / 256.0
    loss, g = net.loss_grad(dims, h2, d[0], d[1], d[2], d[3])
    Lr, gr = NO.loss_and_grad(p, torch.as_tensor(rhs), torch.as_tensor(prev), torch.as_tensor(tgt), mask, h2)
    assert abs(loss - Lr) <= 2e-2 * Lr
    cos = float(g @ gr / (np.linalg.norm(g) * np.linalg.norm(gr)))
    assert cos > 0.99, cos
    assert np.linalg.norm(g - gr) <= 0.1 * np.linalg.norm(gr)
    # every layer's gradient, not only the largest: direction and magnitude
    off = 0
    for cin, cout in NO.LAYERS:
        n = 27 * cin * cout + cout
        a, b = g[off:off + n], gr[off:off + n]
        if np.linalg.norm(b) > 0:
            assert float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b))) > 0.98
            ratio = float(np.linalg.norm(a) / np.linalg.norm(b))
            print("layer %d->%d: norm ratio %.4f" % (cin, cout, ratio))
            assert abs(ratio - 1.0) <= 0.05, ratio  # a scaled layer gradient keeps its cosine, not its norm
        off += n


@pytest.mark.parametrize("layer", range(len(NO.LAYERS)))
def test_net_gradient_finite_differences(bbpp_lib, layer):
    """The GPU gradient of each layer against finite differences of the GPU's
    own loss.  Weights and activations are BF16, so the loss is piecewise
    constant on the scale of a BF16 step and a two-point difference of single
    weights measures rounding, not slope.  The check therefore moves a whole
    layer along its own weights, w -> (1 + t) w (and its bias), at 41 points
    t in [-0.05, 0.05], and takes the slope at t = 0 of a cubic fitted to the
    losses, against g . w.  The rounding leaves noise on the losses, so the bound
    is 10% of |g . w| plus four standard errors of the fitted slope (from the
    fit's residuals): a layer gradient off in sign, by a factor, or missing a
    term fails it, while a layer whose slope is small next to the noise does
    not fail on rounding alone."""
    net = learned.Net(seed=3)
    p = net.get_params()
    nx, ny, nz, nb = 32, 32, 16, 2
    rng = np.random.default_rng(2)
    rhs = rng.normal(size=(nb, nz, ny, nx)).astype(np.float32)
    prev = rng.normal(size=(nb, nz, ny, nx)).astype(np.float32)
    tgt = (0.01 * rhs + 0.001 * rng.normal(size=(nb, nz, ny, nx))).astype(np.float32)
    mask = (rng.random((nz, ny, nx)) < 0.05).astype(np.uint8)
    d = [bbpp.DeviceArray.from_host(a) for a in (rhs, prev, tgt, mask)]
    dims, h2 = (nx, ny, nz), 1.0 / 1024.0
    _, g = net.loss_grad(dims, h2, *d)
    off = sum(27 * ci * co + co for ci, co in NO.LAYERS[:layer])
    ci, co = NO.LAYERS[layer]
    n = 27 * ci * co + co
    v = np.zeros_like(p)
    v[off:off + n] = p[off:off + n]
    ts = np.linspace(-0.05, 0.05, 41)
    losses = []
    for t in ts:
        net.set_params(p + t * v)
        losses.append(net.loss_grad(dims, h2, *d, grads=False)[0])
    net.set_params(p)
    coef, cov = np.polyfit(ts, losses, 3, cov=True)
    slope, se = float(coef[2]), float(np.sqrt(cov[2, 2]))
    an = float(np.dot(g.astype(np.float64), v.astype(np.float64)))
    print("layer %d: fitted slope %.6e +- %.1e, gradient %.6e" % (layer, slope, se, an))
    assert abs(slope - an) <= 0.1 * abs(an) + 4 * se, (slope, se, an)
    assert se < abs(an)  # the fit resolves the slope: the check is not vacuous


def test_net_training_lowers_loss(bbpp_lib):
    data, g, _ = learned.make_ou_dataset(16, 24, nsph=4, rad=2.0, seed=5, tol=1e-10)
    net = learned.Net(seed=4)
    hist = net.train(data, steps=150, batch=4, lr=3e-3)
    assert np.isfinite(hist).all()
    assert hist[-20:].mean() < 0.5 * hist[:5].mean()


def test_net_checkpoint_roundtrip(bbpp_lib, tmp_path):
    net = learned.Net(seed=9)
    p = net.get_params()
    path = str(tmp_path / "net.bin")
    net.save(path)
    other = learned.Net(seed=10)
    assert not np.array_equal(other.get_params(), p)
    other.load(path)
    assert np.array_equal(other.get_params(), p)


def _restrict(a, F):
    nz, ny, nx = a.shape
    return a.reshape(nz // F, F, ny // F, F, nx // F, F).mean(axis=(1, 3, 5))


def _prolong(c, periodic, F):
    """Cell-centred trilinear interpolation by F (F = 2: weights 3/4, 1/4 per
    axis); periodic axes wrap, the others repeat the edge cell.  Axes [z, y, x]."""
    out = c
    for ax in range(3):
        n = out.shape[ax]
        fi = (np.arange(F * n) + 0.5) / F - 0.5
        lo = np.floor(fi).astype(int)
        w = fi - lo
        if periodic[ax]:
            lo_c, hi_c = lo % n, (lo + 1) % n
        else:
            lo_c, hi_c = np.clip(lo, 0, n - 1), np.clip(lo + 1, 0, n - 1)
        sh = [1, 1, 1]
        sh[ax] = -1
        out = np.take(out, lo_c, axis=ax) * (1 - w).reshape(sh) + np.take(out, hi_c, axis=ax) * w.reshape(sh)
    return out


@pytest.mark.parametrize("F", [2, 4])
@pytest.mark.parametrize("bc", ["ppn", "nnn"])
def test_coarse_guess_matches_restatement(bbpp_lib, bc, F):
    """The learned guess on the grid restricted by F: the solver's guess equals
    p_prev + prolong_F(net(restrict_F(r, p_prev, mask)) - restrict_F(p_prev)),
    with the network run directly on numpy-restricted inputs, coarse solid
    cells (at least half the children solid) carrying no correction and fine
    solid cells 0."""
    nx, ny, nz = 32, 16, 48
    g = problems.make_grid(nx, bc, ny=ny, nz=nz)
    rng = np.random.default_rng(5)
    mask = np.zeros((nz, ny, nx), np.uint8)
    mask[6:11, 3:8, 10:17] = 1
    mask[15:17, 9:12, 2:4] = 1
    mask[28:37, 4:12, 16:24] = 1
    rhs = rng.normal(size=(nz, ny, nx))
    rhs[mask == 1] = 0
    prev = rng.normal(size=(nz, ny, nx))
    s = bbpp.Solver(g)
    dmask, drhs, dprev = (bbpp.DeviceArray.from_host(a) for a in (mask, rhs, prev))
    net = learned.Net(seed=4)
    dx = bbpp.DeviceArray((nz, ny, nx), np.float64)
    rep = s.solve(drhs, dx, dmask, tol=1e300, precision=bbpp.FP32_IR, guess=bbpp.GUESS_LEARNED, net=net.handle,
                  prev=dprev.ptr, net_coarsen=F)
    assert rep.iters == 0
    got = dx.download()
    # the same on the host: residual of the warm start (solver's kernel), restriction, network, prolongation
    dr = bbpp.DeviceArray((nz, ny, nx), np.float64)
    s.residual(drhs, dprev, dr, dmask)
    r = dr.download()
    rc, pc = _restrict(r, F), _restrict(prev, F)
    mc = (_restrict(mask.astype(np.float64), F) >= 0.5).astype(np.uint8)
    assert mc.any()
    d_rc, d_pc, d_mc = (bbpp.DeviceArray.from_host(a) for a in (rc, pc, mc))
    d_o = bbpp.DeviceArray(rc.shape, np.float64)
    net.infer((nx // F, ny // F, nz // F), F * F * g.dx * g.dy, d_rc, d_pc, d_mc, d_o)
    corr = np.where(mc == 1, 0.0, d_o.download() - pc)
    periodic = [bc[2] == "p", bc[1] == "p", bc[0] == "p"]
    want = np.where(mask == 1, 0.0, prev + _prolong(corr, periodic, F))
    scale = np.abs(want - prev).max()
    assert scale > 0
    # the solver forms the residual inside its restriction in FP32 arithmetic,
    # this restatement in FP64: the BF16 network inputs may round apart
    assert np.abs(got - want).max() <= 1e-2 * scale
    assert np.abs(got - want).mean() <= 1e-3 * scale
    net.close()


def test_coarsen_rejects_unfit_grids(bbpp_lib):
    """Restriction by F needs every extent a multiple of 4F: 3 is no factor,
    and 24 cells cannot be restricted by 4."""
    g = problems.make_grid(24, "ppn")
    s = bbpp.Solver(g)
    net = learned.Net(seed=4)
    drhs = bbpp.DeviceArray.from_host(np.zeros(g.shape))
    dx = bbpp.DeviceArray(g.shape, np.float64)
    for F in (3, 4):
        with pytest.raises(bbpp.BbppError) as e:
            s.solve(drhs, dx, None, tol=1e300, precision=bbpp.FP32_IR, guess=bbpp.GUESS_LEARNED, net=net.handle,
                    net_coarsen=F)
        assert e.value.status == bbpp.BAD_ARG
    net.close()
    s.close()


def test_learned_guess_gain(bbpp_lib):
    """Train on an OU sequence at 32^3 and compare PCG iterations on held-out
    steps: zero guess (the reference), warm start from p_prev, learned.  The
    learned guess must beat the warm start it starts from, not only zero."""
    data, g, geom = learned.make_ou_dataset(32, 160, nsph=16, rad=2.0, seed=11, tol=1e-10)
    net = learned.Net(seed=1)
    hist = net.train(data, steps=600, batch=4, lr=2e-3)
    assert hist[-50:].mean() < hist[:10].mean()
    s = bbpp.Solver(g)
    mask = data.mask
    res = {"zero": [], "warm": [], "learned": []}
    last = None
    seq = list(learned.ou_sequence_solves(g, mask, mask.download(), 6, seed=999, tol=1e-10))
    for k in range(1, len(seq)):
        rhs, p, _ = seq[k]
        prev = seq[k - 1][1]
        out = learned.iterations_with(s, g, mask, rhs, prev, net, tol=1e-8)
        for key in res:
            res[key].append(out[key][0])
    z, w, l = (np.mean(res[k]) for k in ("zero", "warm", "learned"))
    print("iterations zero %.1f warm %.1f learned %.1f" % (z, w, l))
    assert l < w < z  # the trained guess saves PCG iterations over the warm start, which saves over zero


@pytest.mark.parametrize("coarsen", [1, 2])
def test_guess_graph_replays_match_direct_launches(bbpp_lib, monkeypatch, coarsen):
    """The learned guess runs directly the first time a set of buffers is seen,
    is captured as a CUDA graph the second time and replayed after that.  Three
    guesses with new inputs in the same buffers through that path equal, bit for
    bit, the same guesses launched directly (BBPP_GUESS_GRAPH=0)."""
    nx, ny, nz = 32, 16, 24
    g = problems.make_grid(nx, "ppn", ny=ny, nz=nz)
    rng = np.random.default_rng(17)
    mask = np.zeros((nz, ny, nx), np.uint8)
    mask[6:11, 3:8, 10:17] = 1
    s = bbpp.Solver(g)
    net = learned.Net(seed=4)
    dmask = bbpp.DeviceArray.from_host(mask)
    drhs, dprev = bbpp.DeviceArray((nz, ny, nx), np.float64), bbpp.DeviceArray((nz, ny, nx), np.float64)
    dx = bbpp.DeviceArray((nz, ny, nx), np.float64)
    inputs = []
    for _ in range(3):
        rhs = rng.normal(size=(nz, ny, nx))
        rhs[mask == 1] = 0
        inputs.append((rhs, rng.normal(size=(nz, ny, nx))))
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("BBPP_GUESS_GRAPH", mode)
        res = []
        for rhs, prev in inputs:
            drhs.upload(rhs)
            dprev.upload(prev)
            rep = s.solve(drhs, dx, dmask, tol=1e300, precision=bbpp.FP32_IR, guess=bbpp.GUESS_LEARNED,
                          net=net.handle, prev=dprev.ptr, net_coarsen=coarsen)
            assert rep.iters == 0 and rep.launches > 0
            res.append(dx.download())
        out[mode] = res
    for a, b in zip(out["1"], out["0"]):
        assert np.array_equal(a, b)
    assert not np.array_equal(out["1"][0], out["1"][1])
    net.close()
