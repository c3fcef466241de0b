"""CPU model of the tcgen05 convolution's pipeline (k_conv3_tm in
bluebottle-3.0_gb300/csrc/bbpp_conv_tc.cuh): its three roles (TMA producer,
MMA issuer, epilogue) replayed as generators over the same plane units,
segments, stages and rings, checking that every mbarrier wait finds the
phase it means (no parity alias, no lag), that no interleaving deadlocks,
that every shared-memory, tensor-memory and global address stays in bounds,
and that every output row is written exactly once.  Runs on the CPU; it is the
check of the kernel's index arithmetic that precedes a GPU run, kept as a
test so a change to the kernel's constants or loops is checked the same way."""
import pytest

NST, NACC, NAG, RS, TMEM = 4, 4, 4, 144 * 16, 512


def tyr(cout):
    return 4 if cout <= 16 else 3


class Bar:
    def __init__(self, name, count):
        self.name, self.count, self.arr, self.done = name, count, 0, 0

    def arrive(self):
        self.arr += 1
        if self.arr == self.count:
            self.arr = 0
            self.done += 1


def segs(u0, u1, nz, nxb, nyb):
    u = u0
    while u < u1:
        t = u // nz
        zs = u - t * nz
        ze = min(nz, zs + (u1 - u))
        xb = t % nxb
        t2 = t // nxb
        yield (t2 // nyb, xb, t2 % nyb, zs, ze)
        u += ze - zs


def run(cin, cout, nx, ny, nz, nb, px, py, pz, grid, ldi=None, ci_off=0, ldo=None, co_off=0):
    ldi = ldi or cin
    ldo = ldo or cout
    nch = cin // 16
    T = tyr(cout)
    ROWS = T + 2
    PB = ROWS * RS
    WB = 27 * cout * 32
    WPB = WB // 2
    STAGE = 2 * PB + (WB if nch > 1 else 0)
    SMEM = NST * STAGE + (0 if nch > 1 else WB)
    ACC = T * cout
    ABASE = NACC * ACC
    assert ABASE + NAG * 24 <= TMEM
    nxb, nyb = nx // 128, -(-ny // T)
    units = nb * nyb * nxb * nz
    in_elems = nb * nz * ny * nx * ldi
    out_elems = nb * nz * ny * nx * ldo
    written = set()
    for b in range(grid):
        u0, u1 = b * units // grid, (b + 1) * units // grid
        full = [Bar("full%d" % i, 1) for i in range(NST)]
        ready = [Bar("ready%d" % i, 1) for i in range(NST)]
        empty = [Bar("empty%d" % i, 1) for i in range(NST)]
        abar = [Bar("abar%d" % i, 1) for i in range(NAG)]
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
            if nch == 1:
                wbar.arrive()
            k = 0
            for (vb, xb, yb, zs, ze) in segs(u0, u1, nz, nxb, nyb):
                x0, y0 = xb * 128, yb * T
                ww, ew = px and x0 == 0, px and x0 + 128 == nx
                wbox = 128 if (ww and ew) else (136 if (ww or ew) else 144)
                xs = x0 if ww else x0 - 8
                xoff = 128 if ww else 0
                ywrap = py and (y0 == 0 or y0 + T >= ny)
                for zi in range(zs - 1, ze + 1):
                    for c in range(nch):
                        slot = k % NST
                        sb = slot * STAGE
                        if k >= NST:
                            yield from wait(empty[slot], k // NST - 1)
                        # TMA destinations
                        for kp in range(2):
                            pb = sb + kp * PB + xoff
                            assert pb % 128 == 0
                            # one box of all rows lands them wbox voxels apart: only the
                            # 144-voxel box matches the staged row pitch
                            per_row = wbox != 144 or ywrap
                            pitch = RS if per_row else wbox * 16
                            assert pitch == RS
                            for r in range(ROWS):
                                lo = pb + r * pitch
                                hi = lo + wbox * 16
                                assert lo >= sb and hi <= sb + (kp + 1) * PB, (lo, hi)
                                assert (xoff // 16) + wbox <= 144
                            # coordinates: channel aligned
                            assert (ci_off + 16 * c + 8 * kp) % 8 == 0 and ci_off + 16 * c + 8 * kp + 8 <= ldi
                        if nch > 1:
                            assert sb + 2 * PB + WB <= sb + STAGE and (sb + 2 * PB) % 128 == 0 and WPB % 128 == 0
                        # wrap stores
                        for lane in range(32):
                            side = lane // (2 * ROWS)
                            rem = lane - side * 2 * ROWS
                            wr, wkp = rem >> 1, rem & 1
                            if not px or side > 1 or (x0 != 0 if side == 0 else x0 + 128 != nx):
                                continue
                            dst = sb + wkp * PB + wr * RS + (7 if side == 0 else 136) * 16
                            assert dst >= sb and dst + 16 <= sb + 2 * PB
                            # this slot must not be covered by the tensor copy of that row
                            lo = sb + wkp * PB + xoff + wr * RS
                            hi = lo + wbox * 16
                            assert not (lo <= dst < hi), "wrap slot overlaps tensor copy"
                            gy, gz = y0 - 1 + wr, zi
                            okY = 0 <= gy < ny or py
                            okZ = 0 <= gz < nz or pz
                            if okY and okZ:
                                gy %= ny
                                gz %= nz
                                gx = nx - 1 if side == 0 else 0
                                e = ((((vb * nz + gz) * ny + gy) * nx + gx) * ldi + ci_off + 16 * c + 8 * wkp)
                                assert 0 <= e and e + 8 <= in_elems
                        full[slot].arrive()
                        ready[slot].arrive()
                        k += 1

        def mma():
            if nch == 1:
                yield from wait(wbar, 0)
            k = q0 = arow = 0
            for (vb, xb, yb, zs, ze) in segs(u0, u1, nz, nxb, nyb):
                for zi in range(zs - 1, ze + 1):
                    if zi + 1 < ze:
                        q = q0 + (zi + 1 - zs)
                        if q >= NACC:
                            yield from wait(acce[q % NACC], q // NACC - 1)
                    for c in range(nch):
                        slot = k % NST
                        yield from wait(full[slot], k // NST)
                        yield from wait(ready[slot], k // NST)
                        sb = slot * STAGE
                        wb = sb + 2 * PB if nch > 1 else NST * STAGE
                        for r in range(ROWS):
                            ag = arow % NAG
                            if arow >= NAG:
                                yield from wait(abar[ag], arow // NAG - 1)
                            aslot = ABASE + ag * 24
                            for dx in range(3):
                                st = sb + r * RS + (7 + dx) * 16
                                assert st >= sb and st + 2048 <= sb + (r + 1) * RS and st + PB + 2048 <= sb + 2 * PB
                                assert aslot + 8 * dx + 8 <= TMEM
                            for dz in range(3):
                                zo = zi + 1 - dz
                                if zo < zs or zo >= ze:
                                    continue
                                acc0 = ((q0 + zo - zs) % NACC) * ACC
                                for dy in range(3):
                                    ty = r - dy
                                    if ty < 0 or ty >= T:
                                        continue
                                    for dx in range(3):
                                        tap = dz * 9 + dy * 3 + dx
                                        bst = wb + tap * cout * 16
                                        assert bst + cout * 16 + WPB <= wb + WB
                                        assert wb + WB <= SMEM
                                        assert acc0 + ty * cout + cout <= ABASE
                            abar[ag].arrive()
                            arow += 1
                        empty[slot].arrive()
                        k += 1
                    if zi - 1 >= zs:
                        accf[(q0 + zi - 1 - zs) % NACC].arrive()
                q0 += ze - zs

        def epi():
            q = 0
            for (vb, xb, yb, zs, ze) in segs(u0, u1, nz, nxb, nyb):
                for zo in range(zs, ze):
                    yield from wait(accf[q % NACC], q // NACC)
                    for ty in range(T):
                        y = yb * T + ty
                        if y >= ny:
                            continue
                        for x in (xb * 128, xb * 128 + 127):
                            e = (((vb * nz + zo) * ny + y) * nx + x) * ldo + co_off
                            assert 0 <= e and e + cout <= out_elems
                        written.add((vb, zo, y, xb))
                    for _ in range(128):
                        acce[q % NACC].arrive()
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
                # run this role until it blocks on the same barrier twice
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
    expect = {(vb, z, y, xb) for vb in range(nb) for z in range(nz) for y in range(ny) for xb in range(nxb)}
    assert written == expect, "coverage: %d of %d rows" % (len(written), len(expect))
    return units




CONVS = [(16, 16), (16, 32), (96, 32), (48, 16), (32, 16)]


@pytest.mark.parametrize("cin,cout", CONVS)
@pytest.mark.parametrize("shape", [(128, 5, 3, 2, 1, 1, 0, 152), (256, 2, 5, 2, 0, 1, 1, 152), (128, 5, 3, 2, 1, 1, 0, 3),
                                   (256, 7, 9, 1, 1, 0, 0, 5), (256, 8, 10, 1, 1, 1, 0, 1), (128, 6, 12, 2, 1, 1, 0, 5)])
def test_conv_tc_pipeline_model(cin, cout, shape):
    nx, ny, nz, nb, px, py, pz, grid = shape
    run(cin, cout, nx, ny, nz, nb, px, py, pz, grid)


@pytest.mark.parametrize("cin,cout,ldo,co_off", [(16, 16, 48, 32), (16, 32, 96, 64), (48, 16, 32, 8)])
def test_conv_tc_pipeline_model_channel_windows(cin, cout, ldo, co_off):
    run(cin, cout, 128, 4, 3, 1, 1, 1, 0, 7, ldo=ldo, co_off=co_off)


def test_model_constants_match_kernel():
    """The model's ring sizes and tile shapes are the kernel's (read from its header)."""
    import os
    import re
    src = open(os.path.join(os.path.dirname(__file__), "..", "bluebottle-3.0_gb300", "csrc", "bbpp_conv_tc.cuh")).read()

    def const(name):
        return int(re.search(r"constexpr int %s = ([0-9]+)" % name, src).group(1))

    assert const("TM_NST") == NST and const("TM_NACC") == NACC and const("TM_NAG") == NAG
    assert const("TM_TMEM_COLS") == TMEM
    assert re.search(r"constexpr int TM_RS = 144 \* 16;", src) and RS == 144 * 16
    assert re.search(r"return COUT <= 16 \? 4 : 3;", src) and tyr(16) == 4 and tyr(32) == 3
