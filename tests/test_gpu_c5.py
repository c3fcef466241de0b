"""The combined form at scale (C5 geometry): consecutive solves of an
OU-evolved right-hand-side sequence on the 512^3 grid with 4000 spheres of
radius 5 cells (fixed layout), as the reference's time loop calls its pressure
solve once per inner iteration (src/bluebottle.c:168-232).

Five solves of the sequence, each method carrying its own previous pressure:
the learned guess + FP32 PCG with FP64 reliable updates, plain FP64 PCG
warm-started from its previous solution, and FP32/FP64 PCG warm-started without
the network.  Every solve must reach the 1e-8 true relative residual, and the
methods' solutions must agree with the FP64 one within what two 1e-8 solves
of this operator can differ by.  The network is a small C4-style one trained
here (64^3, 128 spheres of radius 4), enough for the guess's path; the
benchmark trains the full one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_c5_sequence_converges(bbpp_lib):
    import torch
    import bbpp
    from bbpp import learned, problems
    c = problems.CONFIGS["C5"]
    g = problems.make_grid(c["n"], c["bc"])
    cents, radii = problems.place_spheres(g, c["nsph"], c["rad"], c["seed"])
    assert len(cents) == 4000
    s = bbpp.Solver(g)
    dmask = bbpp.DeviceArray(g.shape, np.uint8)
    s.sphere_mask(cents, radii, dmask)
    mask = dmask.download()
    assert 0.01 < mask.mean() < 0.02  # 4000 spheres of ~520 cells in 134M cells

    c4 = problems.CONFIGS["C4"]
    data, _, _ = learned.make_ou_dataset(c4["n"], 64, nsph=c4["nsph"], rad=c4["rad"], seed=c4["seed"])
    net = learned.Net(seed=1)
    net.train(data, steps=200, batch=4, lr=2e-3)

    seq = problems.OUSequenceDevice(g.shape, c["seed"], mask)
    rhs = seq.field()
    torch.cuda.synchronize()
    p0 = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    dv = bbpp.DeviceView.of_tensor  # the solver reads the torch tensors in place
    rep = s.solve(dv(rhs), dv(p0), dmask, tol=c["tol"], precision=bbpp.FP64)
    assert rep.status == bbpp.CONVERGED and rep.true_rel <= c["tol"]
    methods = {"learned_ir": dict(precision=bbpp.FP32_IR, guess=bbpp.GUESS_LEARNED, net=net.handle),
               "fp64_warm": dict(precision=bbpp.FP64, guess=bbpp.GUESS_GIVEN),
               "ir_warm": dict(precision=bbpp.FP32_IR, guess=bbpp.GUESS_GIVEN)}
    state = {k: [p0.clone(), torch.empty_like(p0)] for k in methods}
    for t in range(5):
        rhs = seq.step()
        torch.cuda.synchronize()
        out = {}
        for name, kw in methods.items():
            prev, x = state[name]
            if kw["guess"] == bbpp.GUESS_GIVEN:
                x.copy_(prev)
                torch.cuda.synchronize()
                rep = s.solve(dv(rhs), dv(x), dmask, tol=c["tol"], **kw)
            else:
                rep = s.solve(dv(rhs), dv(x), dmask, tol=c["tol"], prev=prev.data_ptr(), **kw)
            assert rep.status == bbpp.CONVERGED, (name, t, rep.as_dict())
            assert rep.true_rel <= c["tol"] * 1.0001, (name, t, rep.true_rel)
            out[name] = x
            state[name] = [x, prev]
        base = out["fp64_warm"]
        bmax = float(base.abs().max())
        for name in ("learned_ir", "ir_warm"):
            assert float((out[name] - base).abs().max()) <= 1e-5 * bmax, (name, t)
