"""The single-pass scan's look-back (k_scan_lookback in ccl_sort.cu),
checked on a host model: tiles take tickets in order, publish their sum
(flag 1), look back over windows of W predecessors -- nearest first,
stopping at the nearest inclusive prefix (flag 2), waiting while a needed
word is unpublished -- and publish their inclusive prefix.  Whatever order
the tiles' steps interleave in, every tile's exclusive prefix is the sum of
the counts before it, and no tile waits forever (each wait is on a tile
that has already started)."""
import numpy as np
import pytest

AGG, INCL = 1, 2


def _run(counts_per_tile, W, rng):
    T = len(counts_per_tile)
    status = [(0, 0)] * T  # (flag, value)
    agg = [int(c) for c in counts_per_tile]
    prefix = [None] * T
    # per tile: a generator of its steps; the scheduler runs one step of a
    # random started tile at a time (tiles start in ticket order)
    def tile(t):
        status[t] = (INCL if t == 0 else AGG, agg[t])
        yield
        before = 0
        if t > 0:
            top = t - 1
            while True:
                words = [status[j] if j >= 0 else (INCL, 0) for j in range(top, top - W, -1)]
                stop = next((i for i, (f, _) in enumerate(words) if f == INCL), W)
                if any(f == 0 for f, _ in words[:stop + 1]):
                    yield  # a needed word unpublished: re-read the window later
                    continue
                before += sum(v for i, (f, v) in enumerate(words) if i <= stop and f)
                if stop < W:
                    break
                top -= W
        if t > 0:
            status[t] = (INCL, before + agg[t])
        prefix[t] = before
        yield
    gens, started, steps = [], 0, 0
    while True:
        live = [g for g in gens if g is not None]
        if started < T and (not live or rng.random() < 0.5):
            gens.append(tile(started))
            started += 1
            continue
        if not live:
            break
        i = rng.choice([k for k, g in enumerate(gens) if g is not None])
        try:
            next(gens[i])
        except StopIteration:
            gens[i] = None
        steps += 1
        assert steps < 100000  # no wait lasts forever
    return prefix


@pytest.mark.parametrize("W", [1, 4, 32, 256])
def test_lookback_prefixes_for_any_interleaving(W):
    rng = np.random.default_rng(W)
    for trial in range(40):
        T = int(rng.integers(1, 60))
        counts = rng.integers(0, 1000, T)
        got = _run(counts, W, rng)
        want = np.concatenate([[0], np.cumsum(counts)[:-1]])
        assert got == [int(v) for v in want], (trial, T)
