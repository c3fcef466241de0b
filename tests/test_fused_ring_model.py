"""CPU model of the stage ring of the fused FP32 iteration kernel (k1_fused in
bluebottle-3.0_gb300/csrc/bbpp_tma.cu), replaying its schedule for one CTA:
the first min(ns, np) planes are issued up front; step j preps plane j + 1
(waiting on the stage's mbarrier), meets the CTA barrier, refills the stage of
plane j - 2 with plane j - 2 + ns, and runs the stencil of plane j on the stages
of planes j - 1, j and j + 1.  Checked for every ring depth the host allows and
every z-chunk length: each plane is issued once and waited on once with the
phase parity that identifies it, no refill lands on a stage the same step
reads, and the drain waits on exactly the copies still in flight."""
import os
import re

import pytest


def replay(ns, nj):
    np_ = nj + 2  # the chunk's planes plus the halo plane on either side
    stage_of = {}  # plane -> stage holding it
    uses = [0] * ns  # copies issued into each stage so far
    issued, waited = [], []

    def issue(j):
        s = j % ns
        assert j not in stage_of
        stage_of[j] = s
        uses[s] += 1
        issued.append(j)

    def wait(j):
        s = j % ns
        parity = (j // ns) & 1
        # the stage's mbarrier completes one phase per copy; the wait for plane
        # j must find the phase of that copy: (copies into s so far - 1) & 1
        assert stage_of.get(j) == s, "plane %d waited before it was issued" % j
        assert ((uses[s] - 1) & 1) == parity and (uses[s] - 1) == j // ns, (j, uses[s])
        waited.append(j)

    for j in range(min(ns, np_)):
        issue(j)
    wait(0)
    wait(1)
    for j in range(1, nj + 1):
        wait(j + 1)  # prep(j + 1)
        # __syncthreads; then the refill
        if j >= 2 and j - 2 + ns < np_:
            target = j - 2 + ns
            reads = {(j - 1) % ns, j % ns, (j + 1) % ns}
            assert target % ns not in reads, "refill of stage %d while step %d reads it" % (target % ns, j)
            # the plane that stage held (j - 2) is no longer read by any later step
            assert stage_of[j - 2] == target % ns
            issue(target)
        # stencil(j) reads planes j - 1, j, j + 1 from their stages
        for p in (j - 1, j, j + 1):
            assert stage_of[p] == p % ns and p in waited
    assert sorted(issued) == list(range(np_)) and sorted(waited) == list(range(np_))
    drain = list(range(max(0, np_ - ns), np_))
    assert set(drain) <= set(issued) and all(uses[j % ns] - 1 == j // ns for j in drain)


@pytest.mark.parametrize("ns", [4, 5, 6, 7, 8])
def test_fused_ring_schedule(ns):
    for nj in range(1, 70):
        replay(ns, nj)


def test_three_stages_break_the_schedule_as_built():
    """With three stages the first refill would have to wait for the stage of
    plane j - 1, which the stencil of plane j still reads, so plane j + 1 is
    waited on before its copy is issued: the ring needs ns >= 4 as built."""
    with pytest.raises(AssertionError, match="waited before it was issued"):
        replay(3, 10)


def test_model_matches_kernel_source():
    src = open(os.path.join(os.path.dirname(__file__), "..", "bluebottle-3.0_gb300", "csrc", "bbpp_tma.cu")).read()
    body = src[src.index("k1_fused(const GeoL G"):]
    body = body[:body.index("// ------------------------------------------------------------------ host --")]
    assert "if (tid == 0 && j >= 2 && j - 2 + ns < np) issue(j - 2 + ns);" in body
    assert "mbar_wait(&s_full[s], (unsigned int)(j / ns) & 1u, limit)" in body
    assert "const int pre = min(ns, np);" in body
    assert re.search(r"for \(int j = max\(0, np - ns\); j < np; j\+\+\)\s+mbar_wait", body)
    # the host keeps the ring at 4..8 stages
    assert "ns = std::max(4, std::min(8, ns));" in src


# ------------------------------------------------ warp-specialised form ----
def replay_ws(ns, nj, eager):
    """k1_fused_ws: a producer issues plane j into stage j % ns once plane
    j - ns is released (empty barrier, one phase per release); the compute
    warps prep planes 0 and 1, then per step j prep plane j + 1, stencil plane
    j (reads planes j and j + 1; plane j - 1 only at j = 1, later from a
    register) and release plane j (and plane 0 after step 1).  The producer
    runs as far as it can before every consumer wait (eager) or only when the
    consumer would block (lazy).  Checks: no deadlock, every plane issued once
    into a released stage, every wait and release on the phase the kernel's
    parity names, and no read of a plane after its release."""
    np_ = nj + 2
    stage = [None] * ns          # plane a stage holds
    full_done = [0] * ns         # completed phases of each stage's full barrier
    empty_done = [0] * ns        # completed phases of each stage's empty barrier
    released = set()
    nxt = [0]                    # next plane the producer issues

    def produce_one():
        j = nxt[0]
        if j >= np_:
            return False
        s = j % ns
        if j >= ns:
            # the kernel waits for parity (j / ns - 1) & 1: the (j/ns - 1)-th completion
            if empty_done[s] < j // ns:
                return False
            assert empty_done[s] == j // ns and ((empty_done[s] - 1) & 1) == ((j // ns - 1) & 1)
            assert (j - ns) in released, "plane %d issued over unreleased plane %d" % (j, j - ns)
        stage[s] = j
        full_done[s] += 1        # the copy lands (completes one phase)
        nxt[0] += 1
        return True

    def run_producer():
        while produce_one():
            pass

    def wait_full(p):
        if eager:
            run_producer()
        while stage[p % ns] != p:
            assert produce_one(), "deadlock: plane %d never issued" % p
        assert full_done[p % ns] - 1 == p // ns  # parity (p / ns) & 1 names this phase

    def read(p):
        assert p not in released, "plane %d read after release" % p
        assert stage[p % ns] == p

    def release(p):
        released.add(p)
        empty_done[p % ns] += 1

    wait_full(0)
    read(0)
    wait_full(1)
    read(1)
    for j in range(1, nj + 1):
        wait_full(j + 1)
        read(j + 1)                # prep
        for p in (j, j + 1):       # stencil
            read(p)
        if j == 1:
            read(0)
            release(0)
        release(j)
    run_producer()
    assert nxt[0] == np_


@pytest.mark.parametrize("ns", [3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("eager", [True, False])
def test_ws_ring_schedule(ns, eager):
    for nj in range(1, 70):
        replay_ws(ns, nj, eager)


def test_ws_two_stages_deadlock():
    """Two stages: plane 2 needs plane 0's stage, released only after the
    stencil of plane 1, which waits for plane 2 first -- the host keeps ns >= 3."""
    with pytest.raises(AssertionError, match="deadlock"):
        replay_ws(2, 5, False)


def test_ws_model_matches_kernel_source():
    src = open(os.path.join(os.path.dirname(__file__), "..", "bluebottle-3.0_gb300", "csrc", "bbpp_tma.cu")).read()
    body = src[src.index("k1_fused_ws(const GeoL G"):]
    body = body[:body.index("// ------------------------------------------------------------------ host --")]
    assert "if (j >= ns) ok = wait_phase(&s_empty[q], (unsigned int)(j / ns - 1) & 1u, limit);" in body
    assert "if (!wait_phase(&s_full[q], (unsigned int)(j / ns) & 1u, limit)) bad = true;" in body
    assert "if (j == 1) release(0);\n      release(j);" in body
    assert "mbar_init(&s_empty[q], WS_WARPS);" in body
    assert "const float4 b = j == 1 ?" in body
    assert "int wns = std::max(3, std::min(8, env_int(\"BBPP_WS_NS\", 4)));" in src
