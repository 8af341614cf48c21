"""The warp-to-warp hand-over of the LU-SGS row pipelines, simulated on the CPU.

The pipelined sweeps (csrc/k_sweep_common.cuh: HandOff, HandOffN) pass each step's value
from the last row of warp w to the first row of warp w+1 through a one-slot shared buffer
guarded by two named barriers per warp pair, "full" and "empty" (bar.arrive / bar.sync
with a count of 64: the two warps). This test runs the protocol's barrier operations for
every warp count and step count under random interleavings of the warps, with the
hardware's counting semantics (a warp's arrival adds 32 threads; a generation completes at
64 and releases the warps that synced on it), and checks that every run ends and every
consumer reads the value its producer wrote for the previous step.

A CTA that takes several lines in turn (the capped split pipelines, lusgs_cap) repeats the
protocol per line with a CTA barrier between lines (k_sweep_ex32s / k_sweep_eyz32s). Without
that barrier a producer's first put of the next line, which waits on no "empty", can arrive
a second time on "full" before the consumer's last sync of the previous line; the test
shows such runs fail.
"""
import random

import pytest


def _run(nw, nsteps, lines, cta_barrier, seed):
    rnd = random.Random(seed)
    progs = []
    for w in range(nw):
        ops = []
        for line in range(lines):
            for t in range(nsteps):
                if w > 0 and t > 0:  # get: the previous warp's value of step t-1
                    ops += [("sync", ("full", w - 1)), ("read", w - 1, (line, t - 1)), ("arrive", ("empty", w - 1))]
                if w + 1 < nw:  # put: once the next warp has read step t-1
                    if t >= 1:
                        ops.append(("sync", ("empty", w)))
                    ops += [("write", w, (line, t)), ("arrive", ("full", w))]
            if w > 0 and nsteps > 0:  # finish: the last generation of "full"
                ops.append(("sync", ("full", w - 1)))
            if cta_barrier:
                ops.append(("cta",))
        progs.append(ops)
    pc = [0] * nw
    count, waiting, blocked, slot, at_cta = {}, {}, [False] * nw, {}, set()
    while True:
        runnable = [w for w in range(nw) if pc[w] < len(progs[w]) and not blocked[w]]
        if not runnable:
            return "ok" if all(pc[w] >= len(progs[w]) for w in range(nw)) else "deadlock"
        w = rnd.choice(runnable)
        op = progs[w][pc[w]]
        if op[0] in ("sync", "arrive"):
            b = op[1]
            count[b] = count.get(b, 0) + 32
            if op[0] == "sync":
                waiting.setdefault(b, []).append(w)
                blocked[w] = True
            else:
                pc[w] += 1
            if count[b] == 64:  # the generation completes
                count[b] = 0
                for v in waiting.get(b, []):
                    blocked[v] = False
                    pc[v] += 1
                waiting[b] = []
        elif op[0] == "write":
            slot[op[1]] = op[2]
            pc[w] += 1
        elif op[0] == "read":
            if slot.get(op[1]) != op[2]:
                return "wrong value"
            pc[w] += 1
        else:  # CTA barrier
            at_cta.add(w)
            blocked[w] = True
            if len(at_cta) == nw:
                for v in at_cta:
                    blocked[v] = False
                    pc[v] += 1
                at_cta.clear()


@pytest.mark.parametrize("nw", range(1, 9))
def test_handoff_one_line_per_cta(nw):
    for nsteps in range(1, 8):
        for seed in range(25):
            assert _run(nw, nsteps, 1, False, seed * 101 + nsteps) == "ok", (nw, nsteps, seed)


@pytest.mark.parametrize("nw", range(1, 9))
def test_handoff_several_lines_with_cta_barrier(nw):
    for nsteps in range(1, 7):
        for lines in (2, 3):
            for seed in range(20):
                assert _run(nw, nsteps, lines, True, seed * 7919 + nsteps * 13 + lines) == "ok", (nw, nsteps, lines)


def test_handoff_several_lines_without_cta_barrier_fails():
    bad = sum(_run(nw, nsteps, 2, False, seed) != "ok" for nw in (2, 3, 5) for nsteps in (1, 2, 4) for seed in range(30))
    assert bad > 0
