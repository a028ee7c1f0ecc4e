"""GPU parity of the dense-RHS multiply (Y = A.X, FP32 and FP64) and of the
adjoint on the transposed B2SR, against the FP64 oracle, through the C ABI."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_util import REL_TOL, graph_zoo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def zoo(pkg):
    return graph_zoo(pkg)


def spmm_ref(orc, g, X):
    """FP64 CSR SpMM with row-wise |.| sums for the error scale."""
    Y = np.zeros((g.nrows, X.shape[1]))
    S = np.zeros((g.nrows, X.shape[1]))
    rows = np.repeat(np.arange(g.nrows), np.diff(g.rowptr))
    np.add.at(Y, rows, X[g.colind].astype(np.float64))
    np.add.at(S, rows, np.abs(X[g.colind].astype(np.float64)))
    return Y, S


@pytest.mark.parametrize("T", [4, 8, 16, 32])
@pytest.mark.parametrize("k", [1, 16, 32, 64, 100, 128, 200])
def test_spmm_fp32_against_oracle(pkg, orc, cuda, zoo, T, k):
    for name in ("er_4096_d16", "rmat_s12", "hub_40000", "rect_70x333", "empty_rows_only", "dense_96"):
        g = zoo[name]
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        X = np.random.default_rng(k).standard_normal((g.ncols, k)).astype(np.float32)
        Y = A.spmm(torch.from_numpy(X).to(cuda)).cpu().numpy()
        Y64, S = spmm_ref(orc, g, X)
        err = (np.abs(Y[: g.nrows] - Y64) / np.maximum(S, 1e-30)).max(initial=0.0)
        assert err <= REL_TOL, f"{name} T={T} k={k}: rel err {err:.3e}"
        assert np.all(Y[g.nrows:] == 0)
        A.close()


@pytest.mark.parametrize("T", [8, 32])
def test_spmm_matches_oracle_b2sr_order_and_strides(pkg, orc, cuda, zoo, T):
    g = zoo["rmat_s12"]
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
    Xfull = torch.randn(g.ncols, 80, dtype=torch.float64, device=cuda)
    X = Xfull[:, 5:69]  # row stride 80, k = 64: unaligned for vector loads
    Yfull = torch.zeros(A.padded_rows(), 70, dtype=torch.float64, device=cuda)
    Y = Yfull[:, 3:67]
    A.spmm(X, Y)
    want = orc.bmm_f64(T, brp, bci, tiles, X.cpu().numpy())
    np.testing.assert_allclose(Y.cpu().numpy(), want, rtol=1e-12, atol=1e-12)
    assert torch.all(Yfull[:, :3] == 0) and torch.all(Yfull[:, 67:] == 0)
    # accumulate
    Y2 = torch.ones(A.padded_rows(), 64, dtype=torch.float64, device=cuda)
    A.spmm(X.contiguous(), Y2, accumulate=True)
    np.testing.assert_allclose(Y2.cpu().numpy(), want + 1, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("T", [16, 32])
@pytest.mark.parametrize("k", [1, 64, 100])
def test_spmm_dense_tiles_split_steps(pkg, orc, cuda, T, k):
    """Rows with up to 300 sparse columns followed by a dense run of 2048: at
    T = 16 / 32 a 32-tile step of the dense run holds 512 / 1024 items of a
    row, more than a 256-item region, so the row-task kernel appends it in
    lane ranges after flushing what the sparse tiles left; the tile-rows are
    long enough to be cut into segments.  FP32 within the tolerance of the
    FP64 product and FP64 to 1e-11, for the row-task kernel and for the
    merge-path kernel (launch option algorithm = merge)."""
    rng = np.random.default_rng(T * 1000 + k)
    nrows, ncols = 200, 6144
    rows, cols = [], []
    for r in range(nrows):
        sp = rng.choice(4096, size=int(rng.integers(0, 300)), replace=False)
        rows.append(np.full(sp.size + 2048, r))
        cols.append(np.concatenate([sp, np.arange(4096, 6144)]))
    g = pkg.from_edges(np.concatenate(rows), np.concatenate(cols), nrows=nrows, ncols=ncols,
                       drop_self_loops=False)
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    X = rng.standard_normal((ncols, k)).astype(np.float32)
    Y64, S = spmm_ref(orc, g, X)
    for algo in ("auto", "merge"):
        A.set_launch("bin_full_full", algorithm=algo)
        Y = A.spmm(torch.from_numpy(X).to(cuda)).cpu().numpy()
        err = (np.abs(Y[: g.nrows] - Y64) / np.maximum(S, 1e-30)).max(initial=0.0)
        assert err <= REL_TOL, f"{algo} T={T} k={k}: rel err {err:.3e}"
        assert np.all(Y[g.nrows:] == 0)
        Yd = A.spmm(torch.from_numpy(X.astype(np.float64)).to(cuda)).cpu().numpy()
        np.testing.assert_allclose(Yd[: g.nrows], Y64, rtol=1e-11, atol=1e-10)
    A.close()


@pytest.mark.parametrize("T", [4, 8, 32])
def test_adjoint_on_transpose(pkg, orc, cuda, zoo, T):
    g = zoo["rect_70x333"]
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    At = A.transpose()
    dY = np.random.default_rng(1).standard_normal((g.nrows, 48))
    dX = At.spmm(torch.from_numpy(dY).to(cuda)).cpu().numpy()[: g.ncols]
    dense = np.zeros((g.nrows, g.ncols))
    dense[np.repeat(np.arange(g.nrows), np.diff(g.rowptr)), g.colind] = 1
    np.testing.assert_allclose(dX, dense.T @ dY, rtol=1e-12, atol=1e-12)


def test_spmm_is_deterministic(pkg, cuda, zoo):
    g = zoo["hub_40000"]
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    X = torch.randn(g.ncols, 128, device=cuda)
    ys = [A.spmm(X).clone() for _ in range(4)]
    for y in ys[1:]:
        assert torch.equal(y, ys[0])


def test_spmm_column_of_ones_gives_degrees(pkg, cuda, zoo):
    g = zoo["rmat_s12"]
    for T in (4, 16):
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        Y = A.spmm(torch.ones(g.ncols, 33, device=cuda))
        deg = torch.from_numpy(g.degrees().astype(np.float32)).to(cuda)
        assert torch.equal(Y[: g.nrows], deg[:, None].expand(-1, 33))


@pytest.mark.parametrize("T", [4, 8])
@pytest.mark.parametrize("k", [24, 64, 128])
def test_spmm_rhs_blocks_agree(pkg, orc, cuda, zoo, T, k):
    """Every column block (rhs_block: columns per warp pass) gives the FP64
    oracle's product within tolerance, in FP32 and FP64."""
    g = zoo["hub_40000"]
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    X = np.random.default_rng(k).standard_normal((g.ncols, k)).astype(np.float32)
    Y64, S = spmm_ref(orc, g, X)
    for rb in (0, 16, 32, 64, 128):
        A.set_launch("bin_full_full", rhs_block=rb)
        assert A.get_launch("bin_full_full")[5] == rb
        Y = A.spmm(torch.from_numpy(X).to(cuda)).cpu().numpy()
        err = (np.abs(Y[: g.nrows] - Y64) / np.maximum(S, 1e-30)).max(initial=0.0)
        assert err <= REL_TOL, f"T={T} k={k} rhs_block={rb}: rel err {err:.3e}"
        Yd = A.spmm(torch.from_numpy(X.astype(np.float64)).to(cuda)).cpu().numpy()
        np.testing.assert_allclose(Yd[: g.nrows], Y64, rtol=1e-12, atol=1e-12)
    A.close()


@pytest.mark.parametrize("T", [4, 8])
def test_spmm_queue_state_across_calls_and_streams(pkg, orc, cuda, zoo, T):
    """The row-task SpMM keeps its work-queue and long-row arrival counters in
    a per-(matrix, stream) buffer that each launch leaves zeroed: calls with
    one and two column blocks, an SpMV and an accumulating call in between,
    and a first call on a second stream all give the same bits (and the FP64
    oracle's product within the bar)."""
    g = zoo["hub_40000"]
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    rng = np.random.default_rng(T)
    X64 = rng.standard_normal((g.ncols, 64)).astype(np.float32)
    X200 = rng.standard_normal((g.ncols, 200)).astype(np.float32)
    X64d, X200d = torch.from_numpy(X64).to(cuda), torch.from_numpy(X200).to(cuda)
    x = torch.rand(A.ncols, device=cuda)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    s1.wait_stream(torch.cuda.current_stream())
    s2.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s1):
        first = A.spmm(X64d).clone()
        A.spmv_bin_full_full(x)
        wide = A.spmm(X200d).clone()
        acc = A.spmm(X64d).clone()
        A.spmm(X64d, acc, accumulate=True)
        again = A.spmm(X64d).clone()
    with torch.cuda.stream(s2):
        other = A.spmm(X64d).clone()
    torch.cuda.synchronize()
    assert torch.equal(first, again) and torch.equal(first, other)
    for X, Y in ((X64, first), (X200, wide)):
        Y64, S = spmm_ref(orc, g, X)
        err = (np.abs(Y[: g.nrows].cpu().numpy() - Y64) / np.maximum(S, 1e-30)).max(initial=0.0)
        assert err <= REL_TOL, f"T={T} k={X.shape[1]}: rel err {err:.3e}"
    Y64, S = spmm_ref(orc, g, X64)
    err = (np.abs(acc[: g.nrows].cpu().numpy() - 2 * Y64) / np.maximum(2 * S, 1e-30)).max(initial=0.0)
    assert err <= REL_TOL, f"T={T} accumulate: rel err {err:.3e}"
    A.close()


def test_spmm_two_host_threads_two_streams(pkg, cuda, zoo):
    """Two host threads multiplying the same matrix on their own streams at
    once: each stream has its own queue counters and scratch, so both get the
    single-threaded result bit for bit, every time."""
    import threading

    g = zoo["hub_40000"]
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    X = torch.randn(A.ncols, 64, device=cuda)
    want = A.spmm(X).clone()
    torch.cuda.synchronize()
    results, errors = {}, []

    def worker(i):
        try:
            s = torch.cuda.Stream()
            outs = []
            with torch.cuda.stream(s):
                for _ in range(6):
                    outs.append(A.spmm(X).clone())
            s.synchronize()
            results[i] = outs
        except Exception as e:  # reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for outs in results.values():
        for y in outs:
            assert torch.equal(y, want)
    A.close()
