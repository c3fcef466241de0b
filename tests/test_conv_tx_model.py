"""CPU model of the tcgen05 convolution with the x-taps stacked in N
(k_conv3_tx in bluebottle-3.0_gb300/csrc/bbpp_conv_tx.cuh).

Two checks precede any GPU run of the kernel and stay as tests so that a
change to its constants or loops is checked the same way:
  * the pipeline: producer, MMA issuer and epilogue replayed as generators over
    the same plane units, stages and accumulator ring; every mbarrier wait must
    find the phase it means (no parity alias, no lag), no interleaving may
    deadlock, every shared-memory, tensor-memory and global address stays in
    bounds and every output row is written exactly once;
  * the arithmetic: the kernel's schedule (one MMA per staged row, block and
    (dy, dz) with the three x-taps' weights stacked in N, then the epilogue's
    one-voxel shifts with the periodic wrap or zero padding) replayed in FP64
    numpy and compared with a direct 3x3x3 convolution."""
import os
import re

import numpy as np
import pytest

NST, NACC, TMEM = 4, 4, 512


def tyr(cout, nxb):
    return 2 if nxb * cout <= 16 else 1


def accn(cout):
    return 64 if 3 * cout <= 64 else 128


class Bar:
    def __init__(self, name, count):
        self.name, self.count, self.arr, self.done = name, count, 0, 0

    def arrive(self):
        self.arr += 1
        if self.arr == self.count:
            self.arr = 0
            self.done += 1


def segs(u0, u1, nz, nyb):
    u = u0
    while u < u1:
        t = u // nz
        zs = u - t * nz
        ze = min(nz, zs + (u1 - u))
        yield (t // nyb, t % nyb, zs, ze)
        u += ze - zs


def run(cin, cout, nx, ny, nz, nb, px, py, pz, grid, ldi=None, ci_off=0, ldo=None, co_off=0):
    ldi = ldi or cin
    ldo = ldo or cout
    nxb = nx // 128
    assert nx == 128 * nxb and nxb in (1, 2)
    nch = cin // 16
    T = tyr(cout, nxb)
    ROWS = T + 2
    RB = nx * 16
    PB = ROWS * RB
    WB = 27 * cout * 32
    WPB = WB // 2
    STAGE = 2 * PB
    SMEM = NST * STAGE + nch * WB + 1024  # all weights resident after the stages
    AN = accn(cout)
    N3 = 3 * cout
    ACC = T * nxb * AN
    assert N3 <= AN and N3 % 16 == 0 and NACC * ACC <= TMEM
    assert SMEM <= 220 * 1024
    assert STAGE % 128 == 0 and PB % 128 == 0 and WPB % 128 == 0 and RB % 128 == 0
    nyb = -(-ny // T)
    units = nb * nyb * nz
    out_elems = nb * nz * ny * nx * ldo
    written = []
    for b in range(grid):
        u0, u1 = b * units // grid, (b + 1) * units // grid
        full = [Bar("full%d" % i, 1) for i in range(NST)]
        empty = [Bar("empty%d" % i, 1) for i in range(NST)]
        accf = [Bar("accf%d" % i, 1) for i in range(NACC)]
        acce = [Bar("acce%d" % i, 128) for i in range(NACC)]
        wbar = Bar("wbar", 1)

        def wait(bar, n):
            # hardware: succeeds iff (done & 1) != (n & 1); intended: done >= n + 1
            while True:
                hw = (bar.done & 1) != (n & 1)
                want = bar.done >= n + 1
                if hw and not want:
                    raise AssertionError("%s: parity alias, waiting phase %d with %d done" % (bar.name, n, bar.done))
                if want and bar.done > n + 1:
                    raise AssertionError("%s: lag, waiting phase %d with %d done" % (bar.name, n, bar.done))
                if want:
                    return
                yield bar.name

        def producer():
            wbar.arrive()
            k = 0
            for (vb, yb, zs, ze) in segs(u0, u1, nz, nyb):
                y0 = yb * T
                per_row = py and (y0 == 0 or y0 + T >= ny)
                for zi in range(zs - 1, ze + 1):
                    for c in range(nch):
                        slot = k % NST
                        sb = slot * STAGE
                        if k >= NST:
                            yield from wait(empty[slot], k // NST - 1)
                        ch = ci_off + 16 * c
                        assert ch % 8 == 0 and ch + 16 <= ldi
                        for kp in range(2):
                            pb = sb + kp * PB
                            assert pb % 128 == 0
                            for r in range(ROWS):
                                gy = y0 - 1 + r
                                if per_row:  # one box per row, at its wrapped coordinate
                                    gy %= ny
                                    assert 0 <= gy < ny
                                # a periodic y outside the volume is only ever loaded per row
                                assert not py or per_row or 0 <= gy < ny
                                lo, hi = pb + r * RB, pb + (r + 1) * RB
                                assert lo >= sb and hi <= sb + (kp + 1) * PB
                        full[slot].arrive()
                        k += 1

        def mma():
            yield from wait(wbar, 0)
            k = q0 = 0
            for (vb, yb, zs, ze) in segs(u0, u1, nz, nyb):
                for zi in range(zs - 1, ze + 1):
                    if zi + 1 < ze:
                        q = q0 + (zi + 1 - zs)
                        if q >= NACC:
                            yield from wait(acce[q % NACC], q // NACC - 1)
                    for c in range(nch):
                        slot = k % NST
                        yield from wait(full[slot], k // NST)
                        sb = slot * STAGE
                        bd0 = NST * STAGE + c * WB
                        assert bd0 % 128 == 0
                        for r in range(ROWS):
                            for bb in range(nxb):
                                ad = sb + (r * nxb + bb) * 2048
                                # A: 128 voxels x 16 channels, two 8-channel planes PB apart
                                assert ad + 2048 <= sb + PB and ad + PB + 2048 <= sb + 2 * PB
                                for dz in range(3):
                                    zo = zi + 1 - dz
                                    if zo < zs or zo >= ze:
                                        continue
                                    a_s = (q0 + zo - zs) % NACC
                                    for dy in range(3):
                                        ty = r - dy
                                        if ty < 0 or ty >= T:
                                            continue
                                        acc = ((a_s * T + ty) * nxb + bb) * AN
                                        assert acc + N3 <= TMEM
                                        bst = bd0 + (dz * 9 + dy * 3) * cout * 16
                                        # B: the three x-taps' rows, two 8-channel planes WPB apart
                                        assert bst + N3 * 16 <= bd0 + WPB and bst + WPB + N3 * 16 <= bd0 + WB
                                        assert bd0 + WB <= SMEM - 1024 and bd0 >= NST * STAGE
                        empty[slot].arrive()
                        k += 1
                    if zi - 1 >= zs:
                        accf[(q0 + zi - 1 - zs) % NACC].arrive()
                q0 += ze - zs

        def epi():
            q = 0
            for (vb, yb, zs, ze) in segs(u0, u1, nz, nyb):
                for zo in range(zs, ze):
                    a_s = q % NACC
                    yield from wait(accf[a_s], q // NACC)
                    for ty in range(T):
                        for bb in range(nxb):
                            col = ((a_s * T + ty) * nxb + bb) * AN
                            assert col + 3 * cout <= TMEM
                        y = yb * T + ty
                        if y >= ny:
                            continue
                        for x in (0, nx - 1):
                            e = (((vb * nz + zo) * ny + y) * nx + x) * ldo + co_off
                            assert 0 <= e and e + cout <= out_elems and e % 8 == 0
                        written.append((vb, zo, y))
                    for _ in range(128):
                        acce[a_s].arrive()
                    q += 1

        roles = [producer(), mma(), epi()]
        alive = [True] * 3
        steps = 0
        while any(alive):
            progressed = False
            blocked = []
            for i, g in enumerate(roles):
                if not alive[i]:
                    continue
                last = None
                while True:
                    try:
                        w = next(g)
                    except StopIteration:
                        alive[i] = False
                        progressed = True
                        break
                    if w == last:
                        blocked.append((i, w))
                        break
                    last = w
                    progressed = True
                steps += 1
            if not progressed:
                raise AssertionError("deadlock in CTA %d: %s" % (b, blocked))
            if steps > 10 ** 7:
                raise AssertionError("no end")
    expect = sorted((vb, z, y) for vb in range(nb) for z in range(nz) for y in range(ny))
    assert sorted(written) == expect, "coverage: %d of %d rows" % (len(written), len(expect))


def direct_conv(x, w, px, py, pz):
    """x [nz, ny, nx, cin], w [27][cout][cin] with tap = dz 9 + dy 3 + dx;
    out[z, y, x] = sum over taps of w[tap] . in[z + dz - 1, y + dy - 1, x + dx - 1]."""
    nz, ny, nx, _ = x.shape
    out = np.zeros((nz, ny, nx, w.shape[1]))
    pad = [(1, 1)] * 3 + [(0, 0)]
    xp = np.pad(x, pad)
    for ax, p in zip((0, 1, 2), (pz, py, px)):
        if p:
            n = x.shape[ax]
            sl = [slice(None)] * 4
            src = [slice(None)] * 4
            sl[ax], src[ax] = 0, n
            xp[tuple(sl)] = xp[tuple(src)]
            sl[ax], src[ax] = n + 1, 1
            xp[tuple(sl)] = xp[tuple(src)]
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                out += xp[dz:dz + nz, dy:dy + ny, dx:dx + nx] @ w[dz * 9 + dy * 3 + dx].T
    return out


def schedule_conv(x, w, px, py, pz, nxb):
    """The kernel's arithmetic: per staged input row (wrapped or zero-filled as
    its loads are), one product per (dy, dz) with the x-taps stacked in N, then
    the shifts of the epilogue."""
    nz, ny, nx, cin = x.shape
    cout = w.shape[1]
    T = tyr(cout, nxb)
    wst = w.reshape(3, 3, 3 * cout, cin)  # [dz][dy][dx cout + c][k]: the stacked B operand
    out = np.zeros((nz, ny, nx, cout))

    def row(z, y):
        if pz:
            z %= nz
        if not (0 <= z < nz):
            return np.zeros((nx, cin))
        if py and (y < 0 or y >= ny):
            y %= ny
        if not (0 <= y < ny):
            return np.zeros((nx, cin))
        return x[z, y]

    for zo in range(nz):
        for y0 in range(0, ny, T):
            D = np.zeros((T, nx, 3 * cout))
            for zi in (zo - 1, zo, zo + 1):
                dz = zi + 1 - zo  # zo = zi + 1 - dz, as the issuer has it
                for r in range(T + 2):
                    a = row(zi, y0 - 1 + r)
                    for dy in range(3):
                        ty = r - dy
                        if 0 <= ty < T:
                            for bb in range(nxb):
                                v = slice(128 * bb, 128 * bb + 128)
                                D[ty, v] += a[v] @ wst[dz, dy].T
            for ty in range(T):
                if y0 + ty >= ny:
                    continue
                d0, d1, d2 = D[ty, :, :cout], D[ty, :, cout:2 * cout], D[ty, :, 2 * cout:]
                left = np.roll(d0, 1, axis=0)
                right = np.roll(d2, -1, axis=0)
                if not px:
                    left[0] = 0
                    right[-1] = 0
                out[zo, y0 + ty] = left + d1 + right
    return out


CONVS = [(16, 16), (16, 32), (96, 32), (48, 16), (32, 16)]


def variants(cout):
    return [1, 2] if cout == 16 else [1]


@pytest.mark.parametrize("cin,cout", CONVS)
@pytest.mark.parametrize("shape", [(5, 3, 2, 1, 1, 0, 152), (2, 5, 2, 0, 1, 1, 152), (5, 3, 2, 1, 1, 0, 3),
                                   (7, 9, 1, 1, 0, 0, 5), (8, 10, 1, 1, 1, 0, 1), (6, 12, 2, 1, 1, 0, 5)])
def test_conv_tx_pipeline_model(cin, cout, shape):
    ny, nz, nb, px, py, pz, grid = shape
    for nxb in variants(cout):
        run(cin, cout, 128 * nxb, ny, nz, nb, px, py, pz, grid)


@pytest.mark.parametrize("cin,cout,ldo,co_off", [(16, 16, 48, 32), (16, 32, 96, 64), (48, 16, 32, 8)])
def test_conv_tx_pipeline_model_channel_windows(cin, cout, ldo, co_off):
    run(cin, cout, 128, 4, 3, 1, 1, 1, 0, 7, ldo=ldo, co_off=co_off)


@pytest.mark.parametrize("cin,cout,nxb,per", [(16, 16, 1, (1, 1, 0)), (32, 16, 2, (0, 1, 1)), (16, 32, 1, (1, 0, 1)),
                                              (16, 16, 2, (0, 0, 0)), (16, 16, 1, (1, 1, 1))])
def test_conv_tx_schedule_is_the_convolution(cin, cout, nxb, per):
    px, py, pz = per
    rng = np.random.default_rng(cin * 7 + cout + nxb)
    x = rng.standard_normal((3, 5, 128 * nxb, cin))
    w = rng.standard_normal((27, cout, cin))
    ref = direct_conv(x, w, px, py, pz)
    got = schedule_conv(x, w, px, py, pz, nxb)
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


def test_model_constants_match_kernel():
    """The model's ring sizes and tile shapes are the kernel's (read from its header)."""
    src = open(os.path.join(os.path.dirname(__file__), "..", "bluebottle-3.0_gb300", "csrc", "bbpp_conv_tx.cuh")).read()

    def const(name):
        return int(re.search(r"constexpr int %s = ([0-9]+)" % name, src).group(1))

    assert const("TX_NST") == NST and const("TX_NACC") == NACC and const("TX_TMEM_COLS") == TMEM
    assert re.search(r"return NXB \* COUT <= 16 \? 2 : 1;", src)
    assert re.search(r"return 3 \* COUT <= 64 \? 64 : 128;", src)
    assert "(dz * 9 + dy * 3) * COUT * 16" in src
