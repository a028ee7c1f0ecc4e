"""CPU model of the packer's chunked merge (merge_chunks_kernel in
b2sr_pack.cu): a tile-row is cut at the tile-columns of every PACK_CHUNK-th
entry of its longest row; the chunks' tiles, concatenated, must be exactly
the tile-row's tiles in tile-column order."""
from __future__ import annotations

import bisect

import numpy as np
import pytest

PACK_CHUNK = 256


def tiles_of(rows, T, lo=None, hi=None):
    """(tile-column, row words) of a set of CSR rows, tile-columns in [lo, hi)."""
    acc = {}
    for r, cols in enumerate(rows):
        for c in cols:
            tc = c // T
            if (lo is not None and tc < lo) or (hi is not None and tc >= hi):
                continue
            w = acc.setdefault(tc, [0] * T)
            w[r] |= 1 << (T - 1 - c % T)
    return [(tc, tuple(acc[tc])) for tc in sorted(acc)]


def chunked(rows, T):
    lens = [len(c) for c in rows]
    lead = max(range(len(rows)), key=lambda r: (lens[r], -r))
    nk = max(1, -(-lens[lead] // PACK_CHUNK))
    out = []
    for k in range(nk):
        lo_tc = rows[lead][k * PACK_CHUNK] // T if k > 0 else None
        hi_tc = rows[lead][(k + 1) * PACK_CHUNK] // T if k + 1 < nk else None
        part = []
        for cols in rows:  # each lane's [p, e) by lower_bound on the first column of the boundary tile
            p = bisect.bisect_left(cols, lo_tc * T) if lo_tc is not None else 0
            e = bisect.bisect_left(cols, hi_tc * T) if hi_tc is not None else len(cols)
            part.append(cols[p:e])
        out.extend(tiles_of(part, T))
    return out


@pytest.mark.parametrize("T", [4, 8, 16, 32])
@pytest.mark.parametrize("seed", range(6))
def test_chunks_partition_the_tile_row(T, seed):
    rng = np.random.default_rng(seed * 10 + T)
    ncols = int(rng.integers(T, 50000))
    rows = []
    for r in range(T):
        n = int(rng.choice([0, 1, 7, 300, 1000, 3000]))
        if seed % 3 == 0:  # dense clusters: many entries share tile-columns across rows
            base = rng.integers(0, max(1, ncols - 2000))
            cols = np.unique(rng.integers(base, base + 2000, n)) if n else np.zeros(0, np.int64)
        else:
            cols = np.unique(rng.integers(0, ncols, n)) if n else np.zeros(0, np.int64)
        rows.append([int(c) for c in cols])
    assert chunked(rows, T) == tiles_of(rows, T)
