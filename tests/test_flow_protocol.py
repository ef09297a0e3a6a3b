"""A host model of the dataflow Jacobi kernel's scheduling protocol
(k_jacobi_flow in fluid_gb300/csrc/k_pressure.cu), run under many random
interleavings of the blocks' actions:

* items (phase, tile) are claimed in increasing order from one counter;
* a block holds its current item and, once claimed, its next one;
* the next item's boxes are copied (read) only when the up to nine tiles
  around it have published the previous phase -- either mid-sweep, if they
  already have, or after the block published its current tile;
* a tile's results are stored, then published (done[t] = phase + 1).

Checks: no interleaving deadlocks, every copy reads the previous phase of
every neighbour (read after write), and no store overwrites a value a
pending copy of the previous phase still needs (write after read).  The
buffers ping-pong: phase ph reads buffer ph % 2 and writes (ph + 1) % 2.
"""
import random

import pytest


def neighbours(t, ntx, nty):
    ty, tx = divmod(t, ntx)
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            y, x = ty + dy, tx + dx
            if 0 <= y < nty and 0 <= x < ntx:
                yield y * ntx + x


def run(ntx, nty, blocks, nphase, seed):
    rnd = random.Random(seed)
    nt = ntx * nty
    total = nt * nphase
    done = [0] * nt
    buf = [[-1] * nt, [-1] * nt]  # phase whose output each tile slot holds
    readers = [[0] * nt, [0] * nt]  # copies in flight reading each slot
    counter = [0]

    def claim():
        i = counter[0]
        counter[0] += 1
        return i

    def ready(i):
        ph, t = divmod(i, nt)
        return ph == 0 or all(done[n] >= ph for n in neighbours(t, ntx, nty))

    def copy(i):  # the TMA copy of item i's boxes: check and count its reads
        ph, t = divmod(i, nt)
        if ph == 0:
            return
        for n in neighbours(t, ntx, nty):
            assert buf[ph % 2][n] == ph - 1, ("stale read", i, n, buf[ph % 2][n])
            readers[ph % 2][n] += 1

    def land(i):  # the copy is in registers: its reads are over
        ph, t = divmod(i, nt)
        if ph == 0:
            return
        for n in neighbours(t, ntx, nty):
            readers[ph % 2][n] -= 1

    # Block state: cur (item in registers), nxt (claimed), issued (copy of nxt
    # started), stage in {"load", "sweep", "wait"}.
    st = []
    for _ in range(min(blocks, total)):
        i = claim()
        assert ready(i)
        copy(i)
        st.append({"cur": i, "nxt": None, "issued": False, "stage": "load"})
    live = list(range(len(st)))
    steps = 0
    while live:
        steps += 1
        assert steps < 10 ** 7
        cand = [b for b in live
                if st[b]["stage"] in ("load", "sweep")
                or (st[b]["stage"] == "wait" and ready(st[b]["nxt"]))]
        assert cand, "deadlock"
        b = rnd.choice(cand)
        s = st[b]
        if s["stage"] == "load":  # boxes land, next claimed, maybe copied mid-sweep
            land(s["cur"])
            n = claim()
            s["nxt"] = n if n < total else None
            if s["nxt"] is not None and ready(s["nxt"]):
                copy(s["nxt"])
                s["issued"] = True
            s["stage"] = "sweep"
        elif s["stage"] == "sweep":  # sweeps done: store and publish
            ph, t = divmod(s["cur"], nt)
            out = (ph + 1) % 2
            assert readers[out][t] == 0, ("overwrite before read", s["cur"])
            if ph >= 1:
                assert all(done[n] >= ph for n in neighbours(t, ntx, nty))
            buf[out][t] = ph
            done[t] = ph + 1
            if s["nxt"] is None:
                live.remove(b)
            elif s["issued"]:
                s.update(cur=s["nxt"], nxt=None, issued=False, stage="load")
            else:
                s["stage"] = "wait"
        else:  # the pending copy of the next item
            copy(s["nxt"])
            s.update(cur=s["nxt"], nxt=None, issued=False, stage="load")
    assert done == [nphase] * nt
    return steps


@pytest.mark.parametrize("ntx,nty,blocks", [(19, 43, 304), (14, 23, 304), (1, 9, 4), (5, 5, 7),
                                            (3, 4, 12), (25, 7, 175), (11, 15, 165)])
def test_flow_schedule_random_interleavings(ntx, nty, blocks):
    for seed in range(6):
        run(ntx, nty, blocks, 4, seed)
