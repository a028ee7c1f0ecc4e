"""CPU tests of the host graph ingest (include/b2sr_graph.h): canonical form,
determinism, exact edge counts and the Matrix Market reader semantics of the
reference's readMtx (bmv_eval/backend/readMtx.hpp:152-218, 354-422)."""
from __future__ import annotations

import numpy as np
import pytest


def assert_canonical(g, symmetric=True, self_loops=False):
    rp, ci = g.rowptr, g.colind
    assert rp[0] == 0 and rp[-1] == ci.size and np.all(np.diff(rp) >= 0)
    assert ci.size == 0 or (ci.min() >= 0 and ci.max() < g.ncols)
    rows = np.repeat(np.arange(g.nrows), np.diff(rp))
    for i in range(g.nrows):
        seg = ci[rp[i]:rp[i + 1]]
        assert np.all(np.diff(seg) > 0), "rows sorted, no duplicates"
    if not self_loops:
        assert not np.any(rows == ci)
    if symmetric:
        a = set(zip(rows.tolist(), ci.tolist()))
        assert all((c, r) in a for r, c in a)


def test_er_exact_edge_count_and_canonical(pkg):
    g = pkg.erdos_renyi(4096, 16.0, seed=1)
    assert g.nrows == 4096 and g.nnz == 4096 * 16  # exactly m = n*d/2 pairs, mirrored
    assert_canonical(g)
    np.testing.assert_array_equal(g.colind, pkg.erdos_renyi(4096, 16.0, seed=1).colind)
    assert not np.array_equal(g.colind, pkg.erdos_renyi(4096, 16.0, seed=2).colind)


def test_rmat_canonical_deterministic_and_skewed(pkg):
    g = pkg.rmat(12, 16, seed=9)
    assert g.nrows == 4096
    assert_canonical(g)
    h = pkg.rmat(12, 16, seed=9)
    np.testing.assert_array_equal(g.rowptr, h.rowptr)
    np.testing.assert_array_equal(g.colind, h.colind)
    deg = g.degrees()
    # a = 0.57 puts the hubs at low vertex ids (no relabelling)
    assert deg[:64].mean() > 10 * deg[-2048:].mean()
    assert g.nnz < 2 * 16 * 4096  # duplicates and self-loops removed


def test_rmat_quadrant_rule(pkg):
    # scale 1: each edge draws one uniform; u = [r >= a+b], v = [a <= r < a+b or r >= a+b+c]
    a, b, c = 0.57, 0.19, 0.19
    g = pkg.rmat(1, 64, a, b, c, seed=4)
    r = pkg.graphs.uniform_stream(4, 0, 128)
    u = (r >= a + b).astype(int)
    v = (((r >= a) & (r < a + b)) | (r >= a + b + c)).astype(int)
    want = set()
    for uu, vv in zip(u, v):
        if uu != vv:
            want |= {(uu, vv), (vv, uu)}
    rows = np.repeat(np.arange(g.nrows), np.diff(g.rowptr))
    assert set(zip(rows.tolist(), g.colind.tolist())) == want


def test_from_edges_dedup_selfloops_symmetrize(pkg):
    g = pkg.from_edges([0, 0, 0, 1, 2, 2], [1, 1, 0, 2, 2, 0], nrows=3, symmetrize=True)
    assert g.rowptr.tolist() == [0, 2, 4, 6]
    assert g.colind.tolist() == [1, 2, 0, 2, 0, 1]
    k = pkg.from_edges([0, 0, 2], [0, 1, 2], nrows=3, drop_self_loops=False)
    assert k.rowptr.tolist() == [0, 2, 2, 3] and k.colind.tolist() == [0, 1, 2]
    with pytest.raises(ValueError):
        pkg.from_edges([0], [5], nrows=3)


def test_block_diag_offsets(pkg):
    gs = [pkg.erdos_renyi(10, 4.0, seed=s) for s in range(3)]
    bd, offs = pkg.block_diag(gs, align=8)
    assert offs.tolist() == [0, 16, 32, 48]
    assert bd.nrows == 48 and bd.nnz == sum(g.nnz for g in gs)
    for g, o in zip(gs, offs[:-1]):
        np.testing.assert_array_equal(bd.colind[bd.rowptr[o]:bd.rowptr[o + g.nrows]], g.colind + o)
    assert np.all(np.diff(bd.rowptr)[10:16] == 0)


def test_read_mtx_symmetric_pattern(pkg, tmp_path):
    p = tmp_path / "s.mtx"
    p.write_text("%%MatrixMarket matrix coordinate pattern symmetric\n% comment\n4 4 5\n"
                 "2 1\n3 1\n3 3\n4 2\n2 1\n")
    g = pkg.read_mtx(str(p))
    # mirrored, self-loop (3,3) removed, duplicate (2,1) merged
    assert g.rowptr.tolist() == [0, 2, 4, 5, 6]
    assert g.colind.tolist() == [1, 2, 0, 3, 0, 1]
    k = pkg.read_mtx(str(p), drop_self_loops=False)
    assert 2 in k.colind[k.rowptr[2]:k.rowptr[3]].tolist()


def test_read_mtx_general_real_values_become_one(pkg, tmp_path):
    p = tmp_path / "g.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n3 5 3\n1 5 2.5\n3 1 -1\n1 2 7e3\n")
    g = pkg.read_mtx(str(p))
    assert (g.nrows, g.ncols) == (3, 5)
    assert g.rowptr.tolist() == [0, 2, 2, 3]
    assert g.colind.tolist() == [1, 4, 0]


def test_read_mtx_errors(pkg, tmp_path):
    with pytest.raises(ValueError):
        pkg.read_mtx(str(tmp_path / "missing.mtx"))
    bad = tmp_path / "b.mtx"
    bad.write_text("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    with pytest.raises(ValueError):
        pkg.read_mtx(str(bad))
    oob = tmp_path / "o.mtx"
    oob.write_text("%%MatrixMarket matrix coordinate pattern general\n2 2 1\n3 1\n")
    with pytest.raises(ValueError):
        pkg.read_mtx(str(oob))


def test_er_batch_shapes(pkg):
    g, offsets, sizes, degrees = pkg.er_batch(30, 64, 2048, 4, 32, align=32, seed=3)
    assert offsets[0] == 0 and np.all(np.diff(offsets) >= sizes) and np.all(offsets % 32 == 0)
    assert offsets[-1] == g.nrows == g.ncols
    assert sizes.min() >= 64 and sizes.max() <= 2048
    assert degrees.min() >= 4 and degrees.max() <= 32
    rows = np.repeat(np.arange(g.nrows), np.diff(g.rowptr))
    gid_r = np.searchsorted(offsets, rows, side="right") - 1
    gid_c = np.searchsorted(offsets, g.colind, side="right") - 1
    assert np.array_equal(gid_r, gid_c)  # block diagonal
    for i in (0, 7, 29):  # each block: its size, no self-loops, symmetric
        lo = offsets[i]
        blk = rows[(gid_r == i)] - lo
        cb = g.colind[(gid_r == i)] - lo
        assert blk.max(initial=-1) < sizes[i] and np.all(blk != cb)
        e = set(zip(blk.tolist(), cb.tolist()))
        assert all((c, r) in e for r, c in e)
    g2 = pkg.er_batch(30, 64, 2048, 4, 32, align=32, seed=3)[0]
    assert np.array_equal(g.colind, g2.colind)  # deterministic
