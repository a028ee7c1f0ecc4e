"""GPU parity of the multi-frontier Boolean product (32/64 frontiers per vertex
word) against an exact host OR-reduction, and of CUDA-graph capture of the
library's launches."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_util import REL_TOL, full_full_error, graph_zoo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def zoo(pkg):
    return graph_zoo(pkg)


def or_reduce(g, X):
    Y = np.zeros(g.nrows, X.dtype)
    rows = np.repeat(np.arange(g.nrows), np.diff(g.rowptr))
    np.bitwise_or.at(Y, rows, X[g.colind])
    return Y


@pytest.mark.parametrize("T", [4, 8, 16, 32])
@pytest.mark.parametrize("bits", [32, 64])
def test_multi_frontier_or(pkg, cuda, zoo, T, bits):
    npdt, tdt = (np.uint32, torch.int32) if bits == 32 else (np.uint64, torch.int64)
    for name, g in zoo.items():
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        rng = np.random.default_rng(bits + T)
        # frontier f has density ~ 10^U[log10 .001, log10 .05] (multi-source BFS shape)
        dens = 10 ** rng.uniform(np.log10(0.001), np.log10(0.05), size=bits)
        X = np.zeros(g.ncols, npdt)
        for f in range(bits):
            X |= ((rng.random(g.ncols) < dens[f]).astype(npdt) << npdt(f))
        Xt = torch.from_numpy(X.view(np.int32 if bits == 32 else np.int64)).to(cuda)
        Y = A.spmv_multi_bits(Xt).cpu().numpy().view(npdt)
        want = or_reduce(g, X)
        np.testing.assert_array_equal(Y[: g.nrows], want, err_msg=name)
        A.set_launch("bin_full_full", gather="texture")
        Ytx = A.spmv_multi_bits(Xt).cpu().numpy().view(npdt)
        np.testing.assert_array_equal(Ytx[: g.nrows], want, err_msg=name)
        A.set_launch("bin_full_full", gather="ldg")
        assert np.all(Y[g.nrows:] == 0)
        mask = rng.integers(0, 2 ** 31, size=A.padded_rows()).astype(npdt)
        Ym = A.spmv_multi_bits(Xt, mask=torch.from_numpy(mask.view(Xt.cpu().numpy().dtype)).to(cuda))
        np.testing.assert_array_equal(Ym.cpu().numpy().view(npdt)[: g.nrows], want & ~mask[: g.nrows], err_msg=name)
        Y0 = rng.integers(0, 2 ** 31, size=A.padded_rows()).astype(npdt)
        Ya = torch.from_numpy(Y0.view(Xt.cpu().numpy().dtype).copy()).to(cuda)
        A.spmv_multi_bits(Xt, Ya, accumulate=True)
        np.testing.assert_array_equal(Ya.cpu().numpy().view(npdt)[: g.nrows], want | Y0[: g.nrows], err_msg=name)
        A.close()


def test_cuda_graph_capture_and_replay(pkg, orc, cuda, zoo):
    g = zoo["rmat_s12"]
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    x = torch.rand(g.ncols, device=cuda)
    X = torch.randn(g.ncols, 64, device=cuda)
    y = torch.empty(A.padded_rows(), device=cuda)
    Y = torch.empty(A.padded_rows(), 64, device=cuda)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    gr = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        A.spmv_bin_full_full(x, y)  # plans built outside the capture
        A.spmm(X, Y)
    torch.cuda.synchronize()
    with torch.cuda.graph(gr, stream=s):
        A.spmv_bin_full_full(x, y)
        A.spmm(X, Y)
    for _ in range(3):
        x.copy_(torch.rand(g.ncols, device=cuda))
        X.copy_(torch.randn(g.ncols, 64, device=cuda))
        gr.replay()
        torch.cuda.synchronize()
        assert full_full_error(orc, g, x.cpu().numpy(), y.cpu().numpy()) <= REL_TOL
        assert torch.equal(Y, A.spmm(X))
    # a capture on a stream without cached scratch takes pool memory
    gr2 = torch.cuda.CUDAGraph()
    with torch.cuda.graph(gr2):
        A.spmv_bin_full_full(x, y)
    gr2.replay()
    torch.cuda.synchronize()
    assert full_full_error(orc, g, x.cpu().numpy(), y.cpu().numpy()) <= REL_TOL
    A.close()


def test_kernel_timer_records_dominant_kernels(pkg, cuda, zoo):
    """The library's kernel timer records one event pair per multiply while armed,
    skips calls made during stream capture, and stops at its capacity."""
    g = zoo["rmat_s12"]
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    x = torch.rand(g.ncols, device=cuda)
    y = torch.empty(A.padded_rows(), device=cuda)
    X = torch.randn(g.ncols, 16, device=cuda)
    A.spmv_bin_full_full(x, y)
    A.spmm(X)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        A.spmv_bin_full_full(x, y)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with pkg.KernelTimer(3) as t:
        A.spmv_bin_full_full(x, y)
        with torch.cuda.graph(graph, stream=s):
            A.spmv_bin_full_full(x, y)
        A.spmm(X)
        A.set_launch("bin_full_full", algorithm="merge")
        A.spmv_bin_full_full(x, y)
        A.spmv_bin_full_full(x, y)  # past the capacity: not recorded
    assert len(t.ms) == 3
    assert all(0.0 < ms < 1000.0 for ms in t.ms)
    with pkg.KernelTimer(2) as t2:
        pass
    assert t2.ms == []
    A.close()


def test_graph_replay_after_many_vectors(pkg, cuda, zoo):
    """A captured multiply keeps its x gather path valid after many other x
    buffers went through the library (texture handles are never recycled)."""
    g = zoo["rmat_s12"]
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    A.set_launch("bin_full_full", algorithm="rowbin", gather="texture")
    x0 = torch.rand(g.ncols, device=cuda)
    y = torch.empty(A.padded_rows(), device=cuda)
    want = A.spmv_bin_full_full(x0).clone()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        A.spmv_bin_full_full(x0, y)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        A.spmv_bin_full_full(x0, y)
    xs = [torch.rand(g.ncols, device=cuda) for _ in range(40)]
    for x in xs:
        got = A.spmv_bin_full_full(x)
        assert torch.equal(got, A.spmv_bin_full_full(x.clone()))
    y.zero_()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(y, want)
    A.close()


def test_uneven_batch_in_one_captured_launch(pkg, orc, cuda):
    """A block-diagonal batch of uneven Erdos-Renyi graphs (tile-aligned
    offsets): one SpMM over the stack, replayed from a CUDA graph, equals the
    FP64 product, and no graph's rows see another graph's features."""
    g, offsets, sizes, degrees = pkg.er_batch(40, 64, 4096, 4, 32, align=32, seed=7)
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    k = 64
    Xn = np.random.default_rng(1).standard_normal((g.ncols, k)).astype(np.float32)
    X = torch.from_numpy(Xn).to(cuda)
    Y = torch.empty(A.padded_rows(), k, device=cuda)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        A.spmm(X, Y)
    torch.cuda.synchronize()
    gr = torch.cuda.CUDAGraph()
    with torch.cuda.graph(gr, stream=s):
        A.spmm(X, Y)
    Y.zero_()
    gr.replay()
    torch.cuda.synchronize()
    rows = np.repeat(np.arange(g.nrows), np.diff(g.rowptr))
    Y64 = np.zeros((g.nrows, k))
    S = np.zeros((g.nrows, k))
    np.add.at(Y64, rows, Xn[g.colind].astype(np.float64))
    np.add.at(S, rows, np.abs(Xn[g.colind].astype(np.float64)))
    Yh = Y.cpu().numpy()[: g.nrows]
    assert (np.abs(Yh - Y64) / np.maximum(S, 1e-30)).max() <= REL_TOL
    # isolation: features of graph 3 only reach graph 3's rows
    lo, hi = int(offsets[3]), int(offsets[4])
    X2 = torch.zeros_like(X)
    X2[lo:hi] = X[lo:hi]
    Y2 = A.spmm(X2)[: g.nrows].cpu().numpy()
    assert np.all(Y2[:lo] == 0) and np.all(Y2[hi:] == 0)
    np.testing.assert_allclose(Y2[lo:hi], Yh[lo:hi], rtol=0, atol=0)
    A.close()


def test_bin_full_full_matches_cusparse(pkg, cuda, zoo):
    """bin_full_full against cuSPARSE csrmv (torch.mv on a CSR tensor) on the same GPU."""
    for name, g in zoo.items():
        if g.nnz == 0 or g.ncols == 0:
            continue
        A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
        x = torch.rand(g.ncols, device=cuda)
        crow = torch.from_numpy(g.rowptr.astype(np.int64)).to(cuda)
        col = torch.from_numpy(g.colind.astype(np.int64)).to(cuda)
        Acsr = torch.sparse_csr_tensor(crow, col, torch.ones(g.nnz, device=cuda), size=(g.nrows, g.ncols))
        want = torch.mv(Acsr, x)
        got = A.spmv_bin_full_full(x)[: g.nrows]
        scale = torch.mv(Acsr, x.abs()).clamp_min(1e-30)
        assert float(((got - want).abs() / scale).max()) <= 2 * REL_TOL, name
        A.close()
