"""GPU parity of the three multiply variants (and the masked BFS step) against
the oracle, through the C ABI: bit-exact for bits and counts, within REL_TOL
of the FP64 CSR oracle for FP32."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_util import REL_TOL, from_np_words, full_full_error, graph_zoo, to_np_words

pytestmark = pytest.mark.gpu

SHAPES = [(256, 8), (256, 4), (128, 8), (128, 4)]


@pytest.fixture(scope="module")
def zoo(pkg):
    return graph_zoo(pkg)


def _vectors(g, T, seed):
    rng = np.random.default_rng(seed)
    nbc = (g.ncols + T - 1) // T
    x = rng.random(g.ncols, dtype=np.float32)
    xbool = np.zeros(nbc * T, np.float32)
    xbool[: g.ncols] = rng.random(g.ncols) < 0.5
    return x, xbool


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_all_variants_against_oracle(pkg, orc, cuda, zoo, T):
    for name, g in zoo.items():
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
        x, xbool = _vectors(g, T, 11)
        # bin_full_full vs FP64 CSR
        y = A.spmv_bin_full_full(torch.from_numpy(x).to(cuda)).cpu().numpy()
        err = full_full_error(orc, g, x, y)
        assert err <= REL_TOL, f"{name} T={T}: bin_full_full rel err {err:.3e}"
        assert np.all(y[g.nrows:] == 0), name
        # bit inputs
        xb = orc.pack_vec_bits(xbool, T)
        xbt = from_np_words(xb, T, cuda)
        cnt = A.spmv_bin_bin_count(xbt).cpu().numpy()
        np.testing.assert_array_equal(cnt, orc.bmv_bin_bin_count(T, brp, bci, tiles, xb), err_msg=name)
        np.testing.assert_array_equal(cnt[: g.nrows], orc.csr_spmv_count(g.rowptr, g.colind, g.nrows, xbool[: g.ncols]))
        fl = A.spmv_bin_bin_full(xbt).cpu().numpy()
        np.testing.assert_array_equal(fl, orc.bmv_bin_bin_full(T, brp, bci, tiles, xb), err_msg=name)
        yb = to_np_words(A.spmv_bin_bin_bin(xbt), T)
        np.testing.assert_array_equal(yb, orc.bmv_bin_bin_bin(T, brp, bci, tiles, xb), err_msg=name)
        mask = orc.pack_vec_bits((np.random.default_rng(3).random(A.padded_rows()) < 0.5).astype(np.float32), T)
        ym = to_np_words(A.spmv_bin_bin_bin_masked(xbt, from_np_words(mask, T, cuda)), T)
        np.testing.assert_array_equal(ym, orc.bmv_bin_bin_bin_masked(T, brp, bci, tiles, xb, mask), err_msg=name)
        A.close()


@pytest.mark.parametrize("T", [4, 8, 32])
def test_accumulate_semantics(pkg, orc, cuda, zoo, T):
    g = zoo["rmat_s12"]
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
    x, xbool = _vectors(g, T, 5)
    xb = orc.pack_vec_bits(xbool, T)
    xbt = from_np_words(xb, T, cuda)
    y0 = np.random.default_rng(1).random(A.padded_rows(), dtype=np.float32)
    y = torch.from_numpy(y0.copy()).to(cuda)
    A.spmv_bin_full_full(torch.from_numpy(x).to(cuda), y, accumulate=True)
    y64 = orc.csr_spmv_f64(g.rowptr, g.colind, g.nrows, x) + y0[: g.nrows]
    np.testing.assert_allclose(y.cpu().numpy()[: g.nrows], y64, rtol=REL_TOL, atol=1e-5)
    c0 = np.arange(A.padded_rows(), dtype=np.int32)
    c = torch.from_numpy(c0.copy()).to(cuda)
    A.spmv_bin_bin_count(xbt, c, accumulate=True)
    np.testing.assert_array_equal(c.cpu().numpy(), orc.bmv_bin_bin_count(T, brp, bci, tiles, xb, c0, True))
    b0 = orc.pack_vec_bits((np.random.default_rng(2).random(A.padded_rows()) < 0.2).astype(np.float32), T)
    b = from_np_words(b0.copy(), T, cuda)
    A.spmv_bin_bin_bin(xbt, b, accumulate=True)
    np.testing.assert_array_equal(to_np_words(b, T), orc.bmv_bin_bin_bin(T, brp, bci, tiles, xb, b0, True))
    # five accumulating launches, as the reference drivers time them (TEST_TIMES 5)
    y5 = torch.zeros(A.padded_rows(), device=cuda)
    for _ in range(5):
        A.spmv_bin_bin_full(xbt, y5, accumulate=True)
    np.testing.assert_array_equal(y5.cpu().numpy(), 5 * orc.bmv_bin_bin_full(T, brp, bci, tiles, xb))


@pytest.mark.parametrize("threads,items", SHAPES)
def test_launch_shapes_agree(pkg, orc, cuda, zoo, threads, items):
    for name in ("hub_40000", "rmat_s12", "empty_rows_only"):
        g = zoo[name]
        A = pkg.B2SRMatrix.from_graph(g, 8, device=cuda)
        x = np.random.default_rng(9).random(g.ncols, dtype=np.float32)
        xt = torch.from_numpy(x).to(cuda)
        A.set_launch("bin_full_full", threads, items, algorithm="merge")
        assert A.get_launch("bin_full_full")[:2] == (threads, items)
        y = A.spmv_bin_full_full(xt).cpu().numpy()
        assert full_full_error(orc, g, x, y) <= REL_TOL, name
        A.set_launch("bin_full_full", threads, items, ctas_per_sm=1, algorithm="merge")
        y1 = A.spmv_bin_full_full(xt).cpu().numpy()
        assert full_full_error(orc, g, x, y1) <= REL_TOL, name
        # the bit-vector variants on the merge path with the same shape
        brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, 8)
        _, xbool = _vectors(g, 8, 3)
        xb = orc.pack_vec_bits(xbool, 8)
        for v in ("bin_bin_bin", "bin_bin_count"):
            A.set_launch(v, threads, items, algorithm="merge")
        np.testing.assert_array_equal(to_np_words(A.spmv_bin_bin_bin(from_np_words(xb, 8, cuda)), 8),
                                      orc.bmv_bin_bin_bin(8, brp, bci, tiles, xb), err_msg=name)
        np.testing.assert_array_equal(A.spmv_bin_bin_count(from_np_words(xb, 8, cuda)).cpu().numpy(),
                                      orc.bmv_bin_bin_count(8, brp, bci, tiles, xb), err_msg=name)
        A.close()


def test_bin_full_full_is_deterministic(pkg, cuda, zoo):
    g = zoo["hub_40000"]
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    x = torch.from_numpy(np.random.default_rng(0).standard_normal(g.ncols).astype(np.float32)).to(cuda)
    ys = [A.spmv_bin_full_full(x).clone() for _ in range(5)]
    for y in ys[1:]:
        assert torch.equal(y, ys[0])


def test_integer_x_gives_exact_degrees(pkg, cuda, zoo):
    for T in (4, 8, 16, 32):
        g = zoo["rmat_s12"]
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        y = A.spmv_bin_full_full(torch.ones(g.ncols, device=cuda)).cpu().numpy()
        np.testing.assert_array_equal(y[: g.nrows], g.degrees().astype(np.float32))
        A.close()


def test_launch_count_is_reported(pkg, cuda, zoo):
    """One row-binned launch, plus the segment fix-up when a tile-row is cut
    (more than 32 lanes x 4 tiles at T = 8)."""
    g = zoo["er_4096_d16"]
    A = pkg.B2SRMatrix.from_graph(g, 8, device=cuda)
    x = torch.ones(g.ncols, device=cuda)
    A.spmv_bin_full_full(x)  # first call also builds the plan
    A.spmv_bin_full_full(x)
    longest = int(np.diff(A.download()[0]).max())
    assert pkg._lib.load().b2sr_last_launch_count() == (2 if longest > 128 else 1)
    A.close()
    n = 40000  # a star: tile-row 0 holds n/4 tiles, more than one long-row segment
    star = pkg.from_edges(np.zeros(n - 1, np.int32), np.arange(1, n, dtype=np.int32), nrows=n, symmetrize=True)
    S = pkg.B2SRMatrix.from_graph(star, 4, device=cuda)
    y = S.spmv_bin_full_full(torch.ones(n, device=cuda))
    assert pkg._lib.load().b2sr_last_launch_count() == 2
    assert float(y[0]) == n - 1 and float(y[1:n].max()) == 1.0
    S.close()


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_rowbin_and_merge_paths_agree(pkg, orc, cuda, zoo, T):
    for name, g in zoo.items():
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        x = np.random.default_rng(T).standard_normal(g.ncols).astype(np.float32)
        xt = torch.from_numpy(x).to(cuda)
        A.set_launch("bin_full_full", algorithm="rowbin")
        y_rb = A.spmv_bin_full_full(xt).cpu().numpy()
        A.set_launch("bin_full_full", algorithm="rowbin", gather="texture")
        y_tx = A.spmv_bin_full_full(xt).cpu().numpy()
        A.set_launch("bin_full_full", algorithm="merge")
        y_mp = A.spmv_bin_full_full(xt).cpu().numpy()
        assert full_full_error(orc, g, x, y_rb) <= REL_TOL, name
        assert full_full_error(orc, g, x, y_mp) <= REL_TOL, name
        np.testing.assert_array_equal(y_tx, y_rb, err_msg=name)  # same order, other load path
        y0 = np.random.default_rng(1).random(A.padded_rows(), dtype=np.float32)
        A.set_launch("bin_full_full", algorithm="rowbin")
        ya = torch.from_numpy(y0.copy()).to(cuda)
        A.spmv_bin_full_full(xt, ya, accumulate=True)
        y64 = orc.csr_spmv_f64(g.rowptr, g.colind, g.nrows, x)
        scale = orc.csr_spmv_abs_f64(g.rowptr, g.colind, g.nrows, x) + np.abs(y0[: g.nrows])
        err = np.abs(ya.cpu().numpy()[: g.nrows] - (y64 + y0[: g.nrows])) / np.maximum(scale, 1e-30)
        assert err.max(initial=0) <= REL_TOL, name
        A.close()



@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_bit_variants_rowbin_and_merge_agree(pkg, orc, cuda, zoo, T):
    """The row-binned and merge-path forms of the bit-vector variants give the
    same words and counts (plain, accumulating and masked), exactly."""
    for name, g in zoo.items():
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        _, xbool = _vectors(g, T, 5)
        xbt = from_np_words(orc.pack_vec_bits(xbool, T), T, cuda)
        rng = np.random.default_rng(T)
        mask = from_np_words(orc.pack_vec_bits((rng.random(A.padded_rows()) < 0.5).astype(np.float32), T), T, cuda)
        yb0 = from_np_words(orc.pack_vec_bits((rng.random(A.padded_rows()) < 0.3).astype(np.float32), T), T, cuda)
        c0 = torch.from_numpy(rng.integers(0, 50, A.padded_rows()).astype(np.int32)).to(cuda)
        f0 = c0.float()
        res = {}
        for algo in ("merge", "rowbin"):
            for v in ("bin_bin_bin", "bin_bin_count", "bin_bin_full"):
                A.set_launch(v, algorithm=algo)
            yb = yb0.clone()
            A.spmv_bin_bin_bin(xbt, yb, accumulate=True)
            c = c0.clone()
            A.spmv_bin_bin_count(xbt, c, accumulate=True)
            f = f0.clone()
            A.spmv_bin_bin_full(xbt, f, accumulate=True)
            res[algo] = (A.spmv_bin_bin_bin(xbt).clone(), A.spmv_bin_bin_bin_masked(xbt, mask).clone(),
                         A.spmv_bin_bin_count(xbt).clone(), A.spmv_bin_bin_full(xbt).clone(), yb, c, f)
        for a_, b_ in zip(res["merge"], res["rowbin"]):
            assert torch.equal(a_, b_), f"{name} T={T}"
        A.close()


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_full_full_every_gather_path(pkg, orc, cuda, zoo, T):
    """bin_full_full through each x gather path of the row-binned kernel
    (texture segments, ld.global segments, set columns only): within the
    FP32 bar of the FP64 oracle, and all three bitwise equal (each row sums
    its set columns in the same ascending order), accumulate included."""
    for name, g in zoo.items():
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        rng = np.random.default_rng(T)
        x = rng.standard_normal(max(A.ncols, 1)).astype(np.float32)
        xd = torch.from_numpy(x).to(cuda)
        outs = {}
        for mode in ("texture", "ldg", "sparse"):
            A.set_launch("bin_full_full", algorithm="rowbin", gather=mode)
            y = A.spmv_bin_full_full(xd)
            y2 = y.clone()
            A.spmv_bin_full_full(xd, y2, accumulate=True)
            outs[mode] = (y.cpu().numpy(), y2.cpu().numpy())
        base, base2 = outs["texture"]
        assert full_full_error(orc, g, x[: g.ncols], base) <= REL_TOL, name
        for mode, (y, y2) in outs.items():
            assert np.array_equal(y, base), f"{name} {mode}"
            assert np.array_equal(y2, base2), f"{name} {mode} accumulate"
        A.close()
