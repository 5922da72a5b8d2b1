"""The cell sort's fix-up rule, checked on a model of its scatter (host
only).  The scatter claims a cell's slots with one atomic per distinct
cell per warp and round of 32 consecutive particles; the claims of
different warps land in any order.  A cell is flagged for the fix-up when
one of its claims is neither the cell's first nor the direct continuation
of the same warp's claim on the cell in the round before; the fix-up then
sorts the flagged cells' segments by particle number.  The claim: whatever
order the claims land in, the result is the stable sort (ascending particle
number within each cell) -- any disorder leaves a flagged claim in its
cell.  The model follows the kernel's rule (k_scatter in ccl_sort.cu):
kprev/eprev are the cell and the claim end of the previous round's group
that holds its last lane."""
import numpy as np
import pytest

LANES, ROUNDS = 32, 8


def _claims(keys):
    """Per (warp, round): the groups of equal keys, in lane order."""
    out = []
    span = LANES * ROUNDS
    for w0 in range(0, len(keys), span):
        for r in range(ROUNDS):
            lo = w0 + r * LANES
            idx = np.arange(lo, min(lo + LANES, len(keys)))
            if idx.size == 0:
                break
            groups = {}
            for i in idx:
                groups.setdefault(int(keys[i]), []).append(int(i))
            out.append(((w0, r), groups, int(keys[idx[-1]]) if idx[-1] == lo + LANES - 1 else -1))
    return out


def _scatter_and_fix(keys, ncell, rng, order="random"):
    rounds = _claims(keys)
    claims = [(wr, k, items) for wr, groups, _ in rounds for k, items in groups.items()]
    if order == "random":
        perm = rng.permutation(len(claims))
    else:  # each warp's claims in program order, warps interleaved at random
        by_warp = {}
        for j, (wr, _, _) in enumerate(claims):
            by_warp.setdefault(wr[0], []).append(j)
        queues = [list(v) for v in by_warp.values()]
        perm = []
        while queues:
            q = queues[rng.integers(len(queues))]
            perm.append(q.pop(0))
            queues = [q for q in queues if q]
    cursor = np.zeros(ncell, dtype=np.int64)
    b0 = {}
    for j in perm:
        wr, k, items = claims[j]
        b0[(wr, k)] = cursor[k]
        cursor[k] += len(items)
    counts = np.bincount(keys, minlength=ncell)
    off = np.concatenate([[0], np.cumsum(counts)])
    out = np.full(len(keys), -1, dtype=np.int64)
    flagged = np.zeros(ncell, dtype=bool)
    last = {wr: lk for wr, _, lk in rounds}
    groups_of = {wr: g for wr, g, _ in rounds}
    for wr, k, items in claims:
        w0, r = wr
        b = b0[(wr, k)]
        cont = False
        if r > 0 and (w0, r - 1) in groups_of:
            kp = last[(w0, r - 1)]
            if kp == k:
                ep = b0[((w0, r - 1), kp)] + len(groups_of[(w0, r - 1)][kp])
                cont = b == ep
        if b != 0 and not cont:
            flagged[k] = True
        for rank, i in enumerate(items):
            out[off[k] + b + rank] = i
    for k in np.nonzero(flagged)[0]:
        out[off[k]:off[k + 1]] = np.sort(out[off[k]:off[k + 1]])
    return out, flagged


@pytest.mark.parametrize("layout", ["sorted", "near", "random", "dense"])
@pytest.mark.parametrize("order", ["random", "program"])
def test_fixup_rule_gives_the_stable_sort(layout, order):
    rng = np.random.default_rng(["sorted", "near", "random", "dense"].index(layout) * 2
                                + (order == "program"))
    for trial in range(30):
        n = int(rng.integers(1, 3000))
        ncell = int(rng.integers(1, 400))
        if layout == "random":
            keys = rng.integers(0, ncell, n)
        else:
            keys = np.sort(rng.integers(0, ncell, n))
            if layout == "near":  # particles that moved to a neighbouring cell
                mv = rng.random(n) < 0.2
                keys[mv] = np.clip(keys[mv] + rng.integers(-1, 2, mv.sum()), 0, ncell - 1)
            elif layout == "dense":  # a bunch: a few cells hold most particles
                keys = np.sort(rng.choice(min(ncell, 3), n))
        out, flagged = _scatter_and_fix(keys, ncell, rng, order)
        want = np.argsort(keys, kind="stable")
        np.testing.assert_array_equal(out, want)


def test_cell_sorted_input_is_not_flagged_within_a_warp():
    """Particles in cell order: a cell split between rounds of one warp is
    the same warp's continuation and stays unflagged; only cells that span
    two warps can be flagged."""
    rng = np.random.default_rng(5)
    keys = np.repeat(np.arange(200), 8)  # 8 per cell, in order
    _, flagged = _scatter_and_fix(keys, 200, rng, "program")
    span = LANES * ROUNDS
    warp_edges = {int(keys[i]) for i in range(span, len(keys), span)}
    assert set(np.nonzero(flagged)[0]) <= warp_edges
