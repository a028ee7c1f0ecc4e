"""CPU model of the row-binned kernel's group reduction (group_reduce in
b2sr_rowbin.cu): G lanes each hold T partial row sums; after log2(G)
butterfly steps the writer lanes must hold every row's total exactly once."""
from __future__ import annotations

import itertools

import numpy as np
import pytest


def group_reduce(vals):
    """vals: [G, T] per-lane partials -> list of (lane, first_row, values) writes."""
    G, T = vals.shape
    acc = [list(v) for v in vals]
    first = [0] * G
    nv = T
    s = G // 2
    while s >= 1:
        new = [a[:] for a in acc]
        if nv > 1:
            half = nv // 2
            for l in range(G):
                upper = (l & s) != 0
                p = l ^ s
                for k in range(half):
                    keep = acc[l][half + k] if upper else acc[l][k]
                    # the partner gives the half this lane keeps: its upper half if it
                    # is the lower lane, its lower half if it is the upper lane
                    p_upper = (p & s) != 0
                    give_p = acc[p][k] if p_upper else acc[p][half + k]
                    new[l][k] = keep + give_p
                if upper:
                    first[l] += half
            nv = half
        else:
            for l in range(G):
                new[l][0] = acc[l][0] + acc[l ^ s][0]
        acc = new
        s //= 2
    nvals = T // G if T >= G else 1
    writes = []
    for l in range(G):
        writer = T >= G or (l & (G // T - 1)) == 0
        if writer:
            writes.append((l, first[l], acc[l][:nvals]))
    return writes


@pytest.mark.parametrize("T,G", list(itertools.product([4, 8, 16, 32], [1, 2, 4, 8, 16, 32])))
def test_group_reduce_writes_each_row_once(T, G):
    rng = np.random.default_rng(T * 100 + G)
    vals = rng.integers(0, 100, size=(G, T)).astype(np.float64)
    want = vals.sum(axis=0)
    got = np.full(T, np.nan)
    for _, first, v in group_reduce(vals):
        for k, x in enumerate(v):
            assert np.isnan(got[first + k]), "row written twice"
            got[first + k] = x
    np.testing.assert_array_equal(got, want)
