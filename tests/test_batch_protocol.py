"""CPU model of the persistent batch kernel's tile protocol
(2decomp-fft_gb300/csrc/batch_kernel.cu, batch_kernel): every CTA claims
its tickets one tile ahead, waits (thread 0) until every tile of the
descriptor its tile depends on is counted, runs the tile, and counts it at
the start of its next iteration, before it claims or waits for anything
else.  Descriptors are ordered as gbfft_batch's build_desc orders them
(csrc/batch.cu): stage by stage over the grids, each depending on the same
grid's previous pass.

A random scheduler interleaves the CTAs' atomic steps.  Every schedule must
finish with every tile counted, and no tile may start before its
dependency is complete.  A planted mistake (a tile counted only after the
next tile's wait) must deadlock."""
import random

import pytest


def stage_major(grids):
    """Descriptors (tiles, dep) of grids given as lists of per-pass tile
    counts, in build_desc's order."""
    desc, last = [], [-1] * len(grids)
    for s in range(max(len(g) for g in grids)):
        for gi, g in enumerate(grids):
            if s >= len(g):
                continue
            desc.append((g[s], last[gi]))
            last[gi] = len(desc) - 1
    return desc


def run_model(desc, nctas, rng, signal_after_wait=False, max_steps=2_000_000):
    """Returns (finished, counts).  Each CTA is a small state machine whose
    transitions are the kernel's atomic steps."""
    prefix = [0]
    for t, _ in desc:
        prefix.append(prefix[-1] + t)
    total = prefix[-1]
    counter = 0  # the ticket counter (sync[0])
    counts = [0] * len(desc)  # per-descriptor completion counters (sync[2 + i])
    ctas = []
    for _ in range(nctas):
        # the first ticket is claimed before the loop
        ctas.append({"next": counter, "cur": None, "lo": -1, "prev": -1, "state": "top", "work": 0})
        counter += 1

    def desc_of(tk, lo):
        lo = max(lo, 0)
        while prefix[lo + 1] <= tk:
            lo += 1
        return lo

    def dep_ready(d):
        dep = desc[d][1]
        return dep < 0 or counts[dep] >= desc[dep][0]

    def can_step(c):
        if c["state"] == "exit":
            return False
        if c["state"] == "wait":
            if dep_ready(c["lo"]):
                return True
            # the planted mistake: the pending count is given only after the wait
            return False
        return True

    for _ in range(max_steps):
        live = [c for c in ctas if c["state"] != "exit"]
        if not live:
            break
        ready = [c for c in live if can_step(c)]
        if not ready:
            return False, counts  # deadlock: every live CTA waits
        c = rng.choice(ready)
        st = c["state"]
        if st == "top":
            # s_ticket = next; barrier; thread 0 counts the previous tile
            # and claims the next ticket
            c["cur"] = c["next"]
            if c["prev"] >= 0 and not signal_after_wait:
                counts[c["prev"]] += 1
                c["prev"] = -1
            if c["cur"] < total:
                c["next"] = counter
                counter += 1
                c["lo"] = desc_of(c["cur"], c["lo"])
                c["state"] = "wait"
            else:
                if c["prev"] >= 0:
                    counts[c["prev"]] += 1
                    c["prev"] = -1
                c["state"] = "exit"
        elif st == "wait":
            if signal_after_wait and c["prev"] >= 0:
                counts[c["prev"]] += 1
                c["prev"] = -1
            d = c["lo"]
            assert dep_ready(d), "a tile started before its dependency was complete"
            c["state"] = "run"
            c["work"] = rng.randint(1, 4)
        elif st == "run":
            c["work"] -= 1
            if c["work"] == 0:
                c["prev"] = c["lo"]
                c["state"] = "top"
    else:
        raise AssertionError("model did not finish within the step limit")
    return True, counts


def random_grids(rng, n):
    # forward + backward: six passes a grid; a few grids skip an axis (four
    # passes); tile counts from 1 to 40, occasionally a large pass
    grids = []
    for _ in range(n):
        npass = rng.choice([6, 6, 6, 4])
        grids.append([rng.choice([1, 2, 3, 7, 12, 40, 90]) for _ in range(npass)])
    return grids


@pytest.mark.parametrize("seed", range(12))
def test_every_schedule_finishes_and_counts_every_tile(seed):
    rng = random.Random(seed)
    grids = random_grids(rng, rng.randint(1, 9))
    desc = stage_major(grids)
    nctas = rng.choice([1, 2, 3, 5, 8])
    ok, counts = run_model(desc, nctas, rng)
    assert ok, "deadlock with %d CTAs on %s" % (nctas, grids)
    assert counts == [t for t, _ in desc]


def test_one_cta_runs_a_dependent_chain_alone():
    # a single CTA holds the next ticket while it runs the current one: its
    # own count must come before its next wait
    desc = stage_major([[1, 1, 1, 1, 1, 1], [2, 1, 3, 1, 2, 1]])
    ok, counts = run_model(desc, 1, random.Random(0))
    assert ok and counts == [t for t, _ in desc]


def test_counting_after_the_next_wait_deadlocks():
    # planted in the model: a CTA that counts its finished tile only after
    # the next tile's wait waits for itself when that tile depends on it
    desc = stage_major([[1, 1]])
    ok, _ = run_model(desc, 1, random.Random(0), signal_after_wait=True)
    assert not ok


def test_more_ctas_than_tickets():
    desc = stage_major([[1, 1, 1]])
    ok, counts = run_model(desc, 8, random.Random(3))
    assert ok and counts == [1, 1, 1]
