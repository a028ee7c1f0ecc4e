"""Stream capture and the library's cached state: a multiply made during
capture before its plan exists is refused without launching anything (the
plan needs a synchronizing download), and a graph captured earlier stays
valid after later calls on the same stream replaced the matrix's scratch with
a larger buffer (the old buffer is kept until the matrix is freed)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_util import REL_TOL

pytestmark = pytest.mark.gpu

NOT_SUPPORTED = 5


def spmm_f64(g, X):
    """FP64 CSR product (values 1) of every row and its absolute-value scale."""
    rows = np.repeat(np.arange(g.nrows), np.diff(g.rowptr))
    Y = np.zeros((g.nrows, X.shape[1]))
    np.add.at(Y, rows, X[g.colind].astype(np.float64))
    S = np.zeros((g.nrows, X.shape[1]))
    np.add.at(S, rows, np.abs(X[g.colind]).astype(np.float64))
    return Y, S


def test_capture_before_the_plan_exists_is_refused(pkg, cuda):
    lib = pkg._lib.load()
    g = pkg.rmat(12, 16, seed=61)
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    x = torch.rand(A.ncols, device=cuda)
    y = torch.zeros(A.padded_rows(), device=cuda)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        graph.capture_begin()
        rc = lib.b2sr_spmv_bin_full_full(A.handle, x.data_ptr(), y.data_ptr(), 0, s.cuda_stream)
        rc_mm = lib.b2sr_spmm_bin_full_full(A.handle, x.data_ptr(), 1, 1, y.data_ptr(), 1, 0, s.cuda_stream)
        graph.capture_end()
    assert rc == NOT_SUPPORTED and rc_mm == NOT_SUPPORTED
    torch.cuda.synchronize()
    # outside the capture the same call builds its plan; then a capture works
    A.spmv_bin_full_full(x, y)
    torch.cuda.synchronize()
    want = y.clone()
    y.zero_()
    graph2 = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph2, stream=s):
        A.spmv_bin_full_full(x, y)
    graph2.replay()
    torch.cuda.synchronize()
    assert torch.equal(y, want)
    A.close()


def test_transpose_inside_a_capture_is_refused_until_built(pkg, cuda):
    """Building the transpose allocates and synchronizes the stream, so during a
    capture it is refused before anything is recorded; built outside, it is
    the cached handle, which a later capture gets back without any work."""
    import ctypes as C

    lib = pkg._lib.load()
    A = pkg.B2SRMatrix.from_graph(pkg.rmat(12, 16, seed=63), 4, device=cuda)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    torch.cuda.synchronize()
    out = C.c_void_p()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        graph.capture_begin()
        rc = lib.b2sr_matrix_transpose(A.handle, s.cuda_stream, C.byref(out))
        graph.capture_end()
    assert rc == NOT_SUPPORTED and not out.value
    torch.cuda.synchronize()
    At = A.transpose()  # outside the capture: built and cached
    torch.cuda.synchronize()
    graph2 = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        graph2.capture_begin()
        rc2 = lib.b2sr_matrix_transpose(A.handle, s.cuda_stream, C.byref(out))
        graph2.capture_end()
    assert rc2 == 0 and out.value == At.handle.value
    A.close()

@pytest.mark.parametrize("T", [4, 16])
def test_graph_keeps_its_scratch_after_a_larger_eager_call(pkg, cuda, T):
    g = pkg.rmat(12, 16, seed=62)
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    rng = np.random.default_rng(T)
    X64 = rng.standard_normal((A.ncols, 64)).astype(np.float32)
    X128 = rng.standard_normal((A.ncols, 128)).astype(np.float32)
    X64d, X128d = torch.from_numpy(X64).to(cuda), torch.from_numpy(X128).to(cuda)
    Y64 = torch.zeros(A.padded_rows(), 64, device=cuda)
    Y128 = torch.zeros(A.padded_rows(), 128, device=cuda)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        A.spmm(X64d, Y64)  # plan and scratch (sized for k = 64) of stream s
    s.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        A.spmm(X64d, Y64)  # captures the cached k = 64 scratch
    with torch.cuda.stream(s):
        A.spmm(X128d, Y128)  # needs more scratch: a new buffer, the old one kept
    s.synchronize()
    Y64.zero_()
    graph.replay()
    torch.cuda.synchronize()
    for X, Y in ((X64, Y64), (X128, Y128)):
        want, scale = spmm_f64(g, X)
        err = np.abs(Y[: g.nrows].cpu().numpy() - want) / np.maximum(scale, 1e-30)
        assert err.max() <= REL_TOL, f"k={X.shape[1]}: {err.max():.3e}"
    A.close()


@pytest.mark.parametrize("T", [4, 8])
def test_spmm_captured_on_a_fresh_stream(pkg, cuda, T):
    """A capture on a stream that has not run an SpMM yet takes the SpMM
    counter buffer (and scratch) from the graph's own allocations, zeroed in
    the graph: every replay gives the eager result bit for bit."""
    g = pkg.rmat(12, 16, seed=63)
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    X = torch.randn(A.ncols, 64, device=cuda)
    want = A.spmm(X).clone()  # plan built on the default stream
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    Y = torch.zeros(A.padded_rows(), 64, device=cuda)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        A.spmm(X, Y)
    for _ in range(2):
        Y.zero_()
        graph.replay()
        torch.cuda.synchronize()
        assert torch.equal(Y, want)
    A.close()
