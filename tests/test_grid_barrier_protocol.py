"""A host model of the grid-wide barrier of the wavefront SOR's cooperative
kernel (grid_barrier in fluid_gb300/csrc/k_pressure.cu), run under many
random interleavings of the blocks' actions (sequentially consistent: the
kernel orders them with acquire loads, fences and a release add):

* a block reads the generation word g0, then adds 1 to the arrival count;
* the block whose add returns nblocks - 1 resets the count to 0, then adds 1
  to the generation (in that order);
* every other block polls the generation until it differs from g0.

Checks, over several consecutive barriers: no block leaves barrier k before
every block arrived at it, no interleaving deadlocks, and the count is 0
whenever a block that left barrier k arrives at barrier k + 1.
"""
import random

import pytest


def run(nblocks, nbarriers, seed):
    rnd = random.Random(seed)
    count = [0]
    gen = [0]
    arrived = [0] * nbarriers  # blocks that added to the count at barrier k
    # Per block: barrier index, stage in {"read", "add", "reset", "bump", "poll", "done"}.
    st = [{"k": 0, "stage": "read", "g0": None} for _ in range(nblocks)]
    steps = 0
    while any(s["stage"] != "done" for s in st):
        steps += 1
        assert steps < 10 ** 6
        cand = [b for b, s in enumerate(st)
                if s["stage"] in ("read", "add", "reset", "bump")
                or (s["stage"] == "poll" and gen[0] != s["g0"])]
        assert cand, "deadlock"
        b = rnd.choice(cand)
        s = st[b]
        if s["stage"] == "read":
            s["g0"] = gen[0]
            s["stage"] = "add"
        elif s["stage"] == "add":
            old = count[0]
            count[0] += 1
            arrived[s["k"]] += 1
            s["stage"] = "reset" if old == nblocks - 1 else "poll"
        elif s["stage"] == "reset":
            count[0] = 0
            s["stage"] = "bump"
        else:  # "bump", or a poll that sees the new generation: leave
            if s["stage"] == "bump":
                gen[0] += 1
            assert arrived[s["k"]] == nblocks, ("left early", b, s["k"])
            s["k"] += 1
            if s["k"] == nbarriers:
                s["stage"] = "done"
            else:
                s["stage"] = "read"
    assert count[0] == 0 and gen[0] == nbarriers
    assert arrived == [nblocks] * nbarriers


@pytest.mark.parametrize("nblocks", [1, 2, 3, 7, 16])
def test_grid_barrier_random_interleavings(nblocks):
    for seed in range(40):
        run(nblocks, 6, seed)
