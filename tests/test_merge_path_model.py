"""CPU model of the merge-path multiply's work decomposition.

Mirrors, step by step, partition_kernel (b2sr_spmv.cu) and merge_spmv_kernel /
carry_fixup_kernel (b2sr_spmv_impl.cuh) with small CTAs, so the bookkeeping
(33-ary partition search, per-thread merge-path search, segmented carry scan,
run-end fix-ups, CTA carries) is checked against plain row sums on shapes
that stress it: hub rows spanning many threads and CTAs, empty rows, empty
matrices, grids larger than the work.  Values are integers, so sums are exact.
"""
from __future__ import annotations

import numpy as np
import pytest


def partition(rowptr, grid):
    nb = len(rowptr) - 1
    nt = int(rowptr[nb])
    total = nb + nt
    starts = []
    for c in range(grid + 1):
        d = total * c // grid
        lo, hi = max(0, d - nt), min(d, nb)
        while hi - lo > 32:
            span = hi - lo
            probes = [lo + span * (l + 1) // 33 for l in range(32)]
            preds = [rowptr[p + 1] <= d - p - 1 for p in probes]
            t = sum(preds)
            assert preds == [True] * t + [False] * (32 - t), "predicate must be monotone"
            p_last_true = lo + span * t // 33
            p_first_false = lo + span * (t + 1) // 33
            new_lo = p_last_true + 1 if t > 0 else lo
            new_hi = p_first_false if t < 32 else hi
            lo, hi = new_lo, new_hi
        t = sum(1 for l in range(32) if lo + l < hi and rowptr[lo + l + 1] <= d - (lo + l) - 1)
        x = lo + t
        starts.append((x, d - x))
    return starts


def model_spmv(rowptr, tile_vals, grid, threads, items):
    """tile_vals[j] = contribution vector (length T) of tile j.  Returns y[nb, T]."""
    nb = len(rowptr) - 1
    nt = int(rowptr[nb])
    T = tile_vals.shape[1] if tile_vals.ndim == 2 else 1
    y = np.full((nb, T), np.nan)
    starts = partition(rowptr, grid)
    carries = []
    ipc = threads * items
    nwarps = threads // 32
    for cta in range(grid):
        (i0, j0), (ie, je) = starts[cta], starts[cta + 1]
        d_end = ie + je
        carry = np.zeros(T)
        while i0 + j0 < d_end:
            n_items = min(ipc, d_end - (i0 + j0))
            rowend = [int(rowptr[i0 + k + 1]) if i0 + k < nb else nt for k in range(n_items + 1)]

            def search(rd, lo, hi):
                while lo < hi:
                    mid = (lo + hi) >> 1
                    if rowend[mid] <= j0 + rd - mid - 1:
                        lo = mid + 1
                    else:
                        hi = mid
                return lo

            # sub-chunk end first, then per-thread searches bounded by it
            x_end = search(n_items, max(0, n_items - (nt - j0)), min(n_items, nb - i0))
            ntile = n_items - x_end
            keys, accs, ends = [], [], []
            for tid in range(threads):
                rd = min(tid * items, n_items)
                lo = search(rd, max(0, rd - ntile), min(rd, x_end))
                i, j = i0 + lo, j0 + rd - lo
                acc = carry.copy() if tid == 0 else np.zeros(T)
                for _ in range(min(items, n_items - rd)):
                    if j < rowend[i - i0]:
                        acc = acc + tile_vals[j]
                        j += 1
                    else:
                        assert np.isnan(y[i]).all(), "row emitted twice"
                        y[i] = acc
                        acc = np.zeros(T)
                        i += 1
                keys.append(i)
                accs.append(acc)
                ends.append((i, j))
            # warp-level Hillis-Steele segmented scan
            scanned = [a.copy() for a in accs]
            for w in range(nwarps):
                lanes = list(range(w * 32, w * 32 + 32))
                o = 1
                while o < 32:
                    prev = [scanned[t].copy() for t in lanes]
                    for li, t in enumerate(lanes):
                        if li >= o and keys[t - o] == keys[t]:
                            scanned[t] = prev[li - o] + prev[li]
                    o <<= 1
            wkey = [keys[w * 32 + 31] for w in range(nwarps)]
            wfirst = [keys[w * 32] for w in range(nwarps)]
            wacc = [scanned[w * 32 + 31].copy() for w in range(nwarps)]
            final = [s.copy() for s in scanned]
            for t in range(threads):
                w = t // 32
                if w > 0 and keys[t] == wfirst[w]:
                    pre = np.zeros(T)
                    anyp = False
                    for w2 in range(w - 1, -1, -1):
                        if wkey[w2] != keys[t]:
                            break
                        pre = wacc[w2] + pre
                        anyp = True
                        if wfirst[w2] != keys[t]:
                            break
                    if anyp:
                        final[t] = pre + final[t]
            for t in range(threads - 1):
                if keys[t + 1] != keys[t]:
                    assert keys[t] < nb
                    y[keys[t]] = y[keys[t]] + final[t]
            carry = final[threads - 1]
            i0, j0 = ends[threads - 1]
        carries.append((i0, carry))
    for c in range(grid):
        row = carries[c][0]
        if row >= nb or (c > 0 and carries[c - 1][0] == row):
            continue
        tot = carries[c][1].copy()
        c2 = c + 1
        while c2 < grid and carries[c2][0] == row:
            tot = tot + carries[c2][1]
            c2 += 1
        y[row] = y[row] + tot
    return y


def check(rowptr, grid, threads=64, items=3, T=2, seed=0):
    rowptr = np.asarray(rowptr, np.int64)
    nt = int(rowptr[-1])
    rng = np.random.default_rng(seed)
    vals = rng.integers(0, 5, size=(nt, T)).astype(np.float64)
    y = model_spmv(rowptr, vals, grid, threads, items)
    want = np.array([vals[rowptr[i]:rowptr[i + 1]].sum(axis=0) for i in range(len(rowptr) - 1)])
    want = want.reshape(len(rowptr) - 1, T) if len(want) else np.zeros((0, T))
    assert not np.isnan(y).any(), "some row never emitted"
    np.testing.assert_array_equal(y, want)


@pytest.mark.parametrize("grid", [1, 2, 3, 7, 40])
def test_random_rows(grid):
    rng = np.random.default_rng(grid)
    counts = rng.integers(0, 9, size=200)
    check(np.concatenate([[0], np.cumsum(counts)]), grid)


@pytest.mark.parametrize("grid", [1, 3, 11])
def test_hub_row_spans_threads_warps_and_ctas(grid):
    counts = [2, 0, 1500, 0, 0, 3, 700, 1]
    check(np.concatenate([[0], np.cumsum(counts)]), grid, threads=64, items=4)


def test_only_empty_rows_and_empty_matrix():
    check([0] * 300, 4)
    check([0], 1)
    check([0, 0, 5, 5], 10)


def test_power_law_rows_large_partition_search():
    rng = np.random.default_rng(1)
    counts = np.minimum(rng.zipf(1.6, size=5000), 3000)
    check(np.concatenate([[0], np.cumsum(counts)]), 29, threads=64, items=8)


def test_partition_is_balanced_and_monotone():
    rng = np.random.default_rng(2)
    counts = rng.integers(0, 50, size=10000)
    rp = np.concatenate([[0], np.cumsum(counts)])
    grid = 97
    st = partition(rp, grid)
    total = len(counts) + int(rp[-1])
    assert st[0] == (0, 0) and st[-1] == (len(counts), int(rp[-1]))
    for c in range(grid):
        assert st[c][0] <= st[c + 1][0] and st[c][1] <= st[c + 1][1]
        assert sum(st[c + 1]) - sum(st[c]) in (total // grid, total // grid + 1)
        x, j = st[c]
        # merge-path validity: rows before x ended at or before tile j; row x not
        assert x == 0 or rp[x] <= j
        assert x == len(counts) or rp[x + 1] >= j
