"""CPU model of the push direction's work list (push_classify_kernel and
push_scratch_bytes in b2sr_push.cu): every tile-column with a non-zero x word
becomes ceil(len / CH) items of at most CH tiles, placed by per-warp scans and
one counter claim per 256-thread block.  The items must cover the active
columns' tiles exactly once, and their number must stay within the scratch
bound nbc + nt / 32 + 1 for every tile size (CH = 256 at T <= 8, 128 at T = 16,
32 at T = 32).  Also models the push itself on 0/1 tiles: OR and counts over
the transposed tiles equal the row-wise product."""
from __future__ import annotations

import numpy as np
import pytest

CH = {4: 256, 8: 256, 16: 128, 32: 32}
BLOCK = 256


def classify(xw, t_rowptr, T):
    """Items as (first, end, x word) in the order the kernel's scans place them."""
    nbc = len(xw)
    ch = CH[T]
    nblocks = -(-nbc // BLOCK)
    counter = 0
    items = {}
    # blocks claim in any order; model a shuffled claim order
    order = np.random.default_rng(0).permutation(nblocks)
    for blk in order:
        cols = range(blk * BLOCK, min(nbc, (blk + 1) * BLOCK))
        per = []
        for c in cols:
            b, e = t_rowptr[c], t_rowptr[c + 1]
            n = -(-(e - b) // ch) if xw[c] else 0
            per.append((c, b, e, n))
        base = counter
        counter += sum(n for *_, n in per)
        pos = base
        for c, b, e, n in per:
            for k in range(n):
                first = b + k * ch
                items[pos] = (first, min(first + ch, e), xw[c])
                pos += 1
    return [items[i] for i in range(counter)]


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_items_cover_active_tiles_once_within_bound(T):
    rng = np.random.default_rng(T)
    nbc = 3000
    # power-law column lengths, a few hub columns far longer than CH
    lens = np.minimum(rng.zipf(1.6, nbc), 5000).astype(np.int64)
    lens[rng.choice(nbc, 5, replace=False)] = [700, 1300, 2049, 4096, 9000]
    t_rowptr = np.concatenate([[0], np.cumsum(lens)])
    nt = int(t_rowptr[-1])
    xw = (rng.random(nbc) < 0.3).astype(np.int64) * rng.integers(1, 1 << T, nbc)
    items = classify(xw, t_rowptr, T)
    assert len(items) <= nbc + nt // 32 + 1  # push_scratch_bytes' bound
    covered = np.zeros(nt, np.int64)
    for first, end, w in items:
        assert 0 < end - first <= CH[T]
        assert w != 0
        covered[first:end] += 1
    active_tiles = np.zeros(nt, np.int64)
    for c in np.nonzero(xw)[0]:
        active_tiles[t_rowptr[c]:t_rowptr[c + 1]] = 1
    np.testing.assert_array_equal(covered, active_tiles)


@pytest.mark.parametrize("T", [4, 8])
def test_push_over_transpose_equals_pull(T):
    """y bit T-1-r of tile-row tr = OR over active A^T words cc (x bit T-1-cc)
    of bit T-1-r; counts add those bits: the same as the row-wise product."""
    rng = np.random.default_rng(7 + T)
    nrows = ncols = 8 * T
    A = (rng.random((nrows, ncols)) < 0.08).astype(np.int64)
    x = (rng.random(ncols) < 0.2).astype(np.int64)
    want_cnt = A @ x
    nb = nrows // T
    y_bits = np.zeros(nb, np.int64)
    y_cnt = np.zeros(nrows, np.int64)
    for c in range(ncols // T):          # tile-row c of A^T
        xw = sum(int(x[c * T + cc]) << (T - 1 - cc) for cc in range(T))
        if xw == 0:
            continue
        for tr in range(nb):             # its tile in tile-column tr
            blk = A[tr * T:(tr + 1) * T, c * T:(c + 1) * T]
            if not blk.any():
                continue
            words = [sum(int(blk[r, cc]) << (T - 1 - r) for r in range(T)) for cc in range(T)]
            m = 0
            for cc in range(T):
                if (xw >> (T - 1 - cc)) & 1:
                    m |= words[cc]
            y_bits[tr] |= m
            for r in range(T):
                y_cnt[tr * T + r] += sum((words[cc] >> (T - 1 - r)) & 1 for cc in range(T)
                                         if (xw >> (T - 1 - cc)) & 1)
    np.testing.assert_array_equal(y_cnt, want_cnt)
    for tr in range(nb):
        want = sum(int(want_cnt[tr * T + r] > 0) << (T - 1 - r) for r in range(T))
        assert y_bits[tr] == want
