"""Model of the decoupled look-back by which the fused sort's blocks find where their
buckets start (nsg_fused.cuh: lookback_partial, fused_block_minmax, lookback_windows,
lookback_publish).  Every bucket count is final before the kernel starts; block b
reads the words of buckets b-1 .. b-T (its first window) when it starts, combines them
at its first barrier -- the sum of the counts down to the nearest bucket that has
published its inclusive prefix, plus that prefix -- walks further windows only when
none had published, and then publishes its own inclusive prefix.  Over random
schedules (blocks starting in any order, any number resident, publications at any
time between a block's reads) every block must get the exclusive prefix of the counts,
and the walk must end within b / T + 1 windows without waiting on another block."""
import random

import numpy as np
import pytest


def block(b, T, counts, words, out):
    """One block as a sequence of steps; each `yield` lets other blocks run."""
    def window(top):
        # thread t reads bucket top-1-t; a position before bucket 0 reads as published 0
        return [(counts[q], words[q]) if q >= 0 else (0, 1) for q in range(top - 1, top - 1 - T, -1)]

    def combine(win):
        acc = 0
        for cnt, inc1 in win:                  # nearest first
            if inc1:
                return acc + inc1 - 1, True
            acc += cnt
        return acc, False

    first = window(b)                          # read beside the sort's loads
    yield
    acc, found = combine(first)                # at the sort's first barrier
    windows = 1
    top = b - T
    while not found:
        yield
        part, found = combine(window(top))
        acc += part
        top -= T
        windows += 1
    words[b] = acc + counts[b] + 1             # publish
    out[b] = (acc, windows)
    yield


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("T", [4, 32, 256])
def test_lookback_gives_exclusive_prefix(seed, T):
    rng = random.Random(seed * 1000 + T)
    nb = rng.choice([1, 2, 7, 300, 1500])
    counts = np.array([rng.choice([0, 0, 1, 5, 1024, 2048]) for _ in range(nb)], dtype=np.int64)
    words = [0] * nb                           # 0: not published
    out = {}
    resident = rng.choice([1, 3, 64, 608])
    order = list(range(nb))
    # blocks start roughly in index order: local shuffles
    for i in range(0, nb, 8):
        seg = order[i:i + 8]
        rng.shuffle(seg)
        order[i:i + 8] = seg
    pending = [block(b, T, counts, words, out) for b in order]
    running = []
    while pending or running:
        while pending and len(running) < resident:
            running.append(pending.pop(0))
        g = rng.choice(running)
        try:
            next(g)
        except StopIteration:
            running.remove(g)
    excl = np.concatenate(([0], np.cumsum(counts)[:-1]))
    for b in range(nb):
        acc, windows = out[b]
        assert acc == excl[b], (b, acc, excl[b])
        assert windows <= b // T + 1
        assert words[b] == excl[b] + counts[b] + 1
