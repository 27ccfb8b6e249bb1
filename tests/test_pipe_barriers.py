"""The named-barrier protocol of the pipelined correlator helpers with two helper sets
(fs_pimc.cuh, FS_PSETS = 2), run as a model on the CPU: every thread group's sequence of
barrier operations, for every operator-run count, completes (no group waits forever) under
every scheduling order, and each snapshot buffer is written only after its previous
measurement was read.

Barrier semantics (PTX bar.sync / bar.arrive with a thread count): an operation adds its
group's threads to the barrier's current phase; the phase completes when the count is
reached; sync blocks its group until the phase it joined completes, arrive does not."""
import itertools
import random

import pytest

FULL = {0: 3, 1: 5}
EMPTY = {0: 4, 1: 6}


def mover_ops(R):
    ops = []
    for run in range(R):
        s = run & 1
        if run >= 2:
            ops.append(("sync", EMPTY[s], ("read_done", run - 2)))
        ops.append(("write", s, run))
        ops.append(("arrive", FULL[s], None))
    for m in range(max(R - 2, 0), R):
        ops.append(("sync", EMPTY[m & 1], ("read_done", m)))
    ops.append(("sync", 0, None))  # the final __syncthreads
    return ops


def helper_ops(R, hs):
    ops = []
    for run in range(hs, R, 2):
        ops.append(("sync", FULL[hs], None))
        ops.append(("read", hs, run))
        ops.append(("arrive", EMPTY[hs], None))
        ops.append(("sync", 7 + hs, None))  # the set's own barrier before its lag sums
    ops.append(("sync", 0, None))
    return ops


def simulate(R, order_seed):
    groups = {"m": mover_ops(R), "h0": helper_ops(R, 0), "h1": helper_ops(R, 1)}
    members = {0: {"m", "h0", "h1"}, 3: {"m", "h0"}, 4: {"m", "h0"}, 5: {"m", "h1"}, 6: {"m", "h1"},
               7: {"h0"}, 8: {"h1"}}
    pc = {g: 0 for g in groups}
    waiting = {}                      # group -> (barrier, phase)
    arrived = {b: set() for b in members}
    phase = {b: 0 for b in members}
    buf = {0: None, 1: None}          # the measurement each snapshot holds
    reads = set()
    rng = random.Random(order_seed)
    steps = 0
    while True:
        steps += 1
        assert steps < 100000
        runnable = [g for g in groups if pc[g] < len(groups[g]) and g not in waiting]
        if not runnable:
            if all(pc[g] == len(groups[g]) for g in groups) and not waiting:
                return True
            return False          # deadlock: every unfinished group waits
        g = rng.choice(runnable)
        op, arg, extra = groups[g][pc[g]]
        pc[g] += 1
        if op == "write":
            prev = buf[arg]
            assert prev is None or prev in reads, ("snapshot overwritten before it was read", arg, prev)
            buf[arg] = extra
        elif op == "read":
            assert buf[arg] == extra, ("helper read the wrong measurement", arg, buf[arg], extra)
            reads.add(extra)
        else:
            b = arg
            assert g not in arrived[b], ("a group joined one barrier phase twice", g, b)
            arrived[b].add(g)
            if op == "sync":
                waiting[g] = (b, phase[b])
            if arrived[b] == members[b]:
                arrived[b] = set()
                phase[b] += 1
                for w, (wb, ph) in list(waiting.items()):
                    if wb == b and ph == phase[b] - 1:
                        del waiting[w]


@pytest.mark.parametrize("R", range(1, 9))
def test_two_set_protocol_completes_under_any_schedule(R):
    for seed in range(300):
        assert simulate(R, seed), (R, seed)
