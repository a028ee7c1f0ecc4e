"""Parity at the benchmark's full size: R-MAT scale 20 (2^20 vertices, edge
factor 16, a/b/c = .57/.19/.19, seed 1; 31.4 M directed edges), every variant
through the C ABI against the oracle's CSR products on the same inputs (the
oracle's C loops take well under a second at this size), plus properties that
hold at any size: x = 1 gives the degrees exactly, the FP32 product is linear
within the FP32 tolerance, the push and pull directions agree bit for bit, and
the packed structure holds every edge once."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_util import REL_TOL, full_full_error

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rmat20(pkg):
    return pkg.rmat(20, 16, 0.57, 0.19, 0.19, 1)


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_rmat20_all_variants_against_oracle(pkg, orc, cuda, rmat20, T):
    g = rmat20
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    assert A.nnz == g.nnz  # every edge packed once
    rng = np.random.default_rng(20 + T)
    # bin_full_full: FP32 against the FP64 CSR product
    x = rng.random(g.ncols, dtype=np.float32)
    y = A.spmv_bin_full_full(torch.from_numpy(x).to(cuda)).cpu().numpy()
    err = full_full_error(orc, g, x, y)
    assert err <= REL_TOL, f"T={T}: bin_full_full rel err {err:.3e}"
    assert np.all(y[g.nrows:] == 0)
    # x = 1: the degrees, exactly
    deg = A.spmv_bin_full_full(torch.ones(g.ncols, device=cuda))[: g.nrows].cpu().numpy()
    np.testing.assert_array_equal(deg, np.diff(g.rowptr).astype(np.float32))
    # bit variants at the BFS-step density: counts and OR exactly
    xbool = np.zeros(A.nblockcols * T, np.float32)
    xbool[: g.ncols] = rng.random(g.ncols) < 0.01
    xbits = A.pack_bits(torch.from_numpy(xbool).to(cuda), A.nblockcols * T)
    want_cnt = orc.csr_spmv_count(g.rowptr, g.colind, g.nrows, xbool[: g.ncols])
    cnt = A.spmv_bin_bin_count(xbits).cpu().numpy()
    np.testing.assert_array_equal(cnt[: g.nrows], want_cnt)
    assert np.all(cnt[g.nrows:] == 0)
    full = A.spmv_bin_bin_full(xbits).cpu().numpy()
    np.testing.assert_array_equal(full[: g.nrows], want_cnt.astype(np.float32))
    yb = A.unpack_bits(A.spmv_bin_bin_bin(xbits), A.padded_rows()).cpu().numpy()
    np.testing.assert_array_equal(yb[: g.nrows] != 0, want_cnt != 0)
    # push and auto equal the pull bit for bit (masked step included)
    visited = A.pack_bits(torch.from_numpy((rng.random(A.padded_rows()) < 0.5).astype(np.float32)).to(cuda),
                          A.padded_rows())
    pull = (A.spmv_bin_bin_bin(xbits).clone(), A.spmv_bin_bin_bin_masked(xbits, visited).clone(),
            A.spmv_bin_bin_count(xbits).clone())
    for direction in ("push", "auto"):
        for v in ("bin_bin_bin", "bin_bin_count"):
            A.set_launch(v, direction=direction)
        got = (A.spmv_bin_bin_bin(xbits), A.spmv_bin_bin_bin_masked(xbits, visited), A.spmv_bin_bin_count(xbits))
        for a, b in zip(got, pull):
            assert torch.equal(a, b), direction
    A.close()


def test_rmat20_linearity_and_determinism(pkg, cuda, rmat20):
    """A(x1 + x2) = A x1 + A x2 within the parity bar (each product within
    REL_TOL of its row's absolute sum; x >= 0 here, so the row sums are the
    products themselves), and repeated calls give identical bits."""
    g = rmat20
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    gen = torch.Generator(device=cuda).manual_seed(5)
    x1 = torch.rand(g.ncols, device=cuda, generator=gen)
    x2 = torch.rand(g.ncols, device=cuda, generator=gen)
    y1 = A.spmv_bin_full_full(x1)
    y2 = A.spmv_bin_full_full(x2)
    y12 = A.spmv_bin_full_full(x1 + x2)
    bound = 2.0 * REL_TOL * (y1 + y2) + 1e-30
    assert bool(((y12 - (y1 + y2)).abs() <= bound).all())
    again = A.spmv_bin_full_full(x1)
    assert torch.equal(y1, again)
    A.close()


def test_rmat20_adjoint_is_the_transpose(pkg, cuda, rmat20):
    """<A x, z> = <x, A^T z> in FP64 on the full graph (the FP64 dense-RHS
    product with k = 4 on A and on its cached transpose)."""
    g = rmat20
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    At = A.transpose()
    gen = torch.Generator(device=cuda).manual_seed(9)
    x = torch.rand(A.ncols, 4, device=cuda, dtype=torch.float64, generator=gen)
    z = torch.rand(A.padded_rows(), 4, device=cuda, dtype=torch.float64, generator=gen)
    ax = A.spmm(x)
    atz = At.spmm(z[: At.ncols].contiguous())
    lhs = (ax[: g.nrows] * z[: g.nrows]).sum(0)
    rhs = (x[: g.ncols] * atz[: g.ncols]).sum(0)
    torch.testing.assert_close(lhs, rhs, rtol=1e-12, atol=0.0)
    A.close()



@pytest.mark.parametrize("T", [4, 16])
def test_rmat20_transpose_of_symmetric_is_itself(pkg, cuda, rmat20, T):
    """The symmetrised graph is its own transpose, so the device transpose
    (three 8-bit digit passes over the 262,144 tile-columns at T = 4, two over
    65,536 at T = 16) must give back A's rowptr, colind and tiles exactly."""
    A = pkg.B2SRMatrix.from_graph(rmat20, T, device=cuda)
    At = A.transpose()
    for a, b in zip(A.download(), At.download()):
        np.testing.assert_array_equal(a, b)
    A.close()

@pytest.fixture(scope="module")
def rmat18(pkg):
    return pkg.rmat(18, 16, 0.57, 0.19, 0.19, 1)


@pytest.mark.parametrize("bits", [32, 64])
def test_rmat18_multi_frontier_exact(pkg, cuda, rmat18, bits):
    """The multi-source BFS configuration at full size: 32 or 64 frontiers of
    0.1-5% density on R-MAT scale 18; Y = OR of the neighbours' words, exactly
    (numpy bitwise OR over the CSR), at the autotuned T = 4 and at T = 8."""
    g = rmat18
    npdt = np.uint32 if bits == 32 else np.uint64
    rng = np.random.default_rng(bits)
    dens = 10 ** rng.uniform(np.log10(0.001), np.log10(0.05), size=bits)
    X = np.zeros(g.ncols, npdt)
    for f in range(bits):
        X |= ((rng.random(g.ncols) < dens[f]).astype(npdt) << npdt(f))
    want = np.zeros(g.nrows, npdt)
    rows = np.repeat(np.arange(g.nrows), np.diff(g.rowptr))
    np.bitwise_or.at(want, rows, X[g.colind])
    Xt = torch.from_numpy(X.view(np.int32 if bits == 32 else np.int64)).to(cuda)
    for T in (4, 8):
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        Y = A.spmv_multi_bits(Xt).cpu().numpy().view(npdt)
        np.testing.assert_array_equal(Y[: g.nrows], want, err_msg=f"T={T}")
        A.close()


def test_rmat18_spmm_k64_against_fp64(pkg, cuda, rmat18):
    """The FP32 feature-block configuration at full size: Y = A.X with X
    [2^18, 64] ~ N(0,1), within REL_TOL of the FP64 product per row, scaled by
    the row's absolute sum (the same bar as the single-vector product)."""
    sp = pytest.importorskip("scipy.sparse")
    g = rmat18
    X = np.random.default_rng(64).standard_normal((g.ncols, 64)).astype(np.float32)
    X64 = X.astype(np.float64)
    A64 = sp.csr_matrix((np.ones(g.nnz), g.colind, g.rowptr), shape=(g.nrows, g.ncols))
    want = A64 @ X64
    scale = A64 @ np.abs(X64)
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    Y = A.spmm(torch.from_numpy(X).to(cuda)).cpu().numpy()
    err = np.abs(Y[: g.nrows] - want) / np.maximum(scale, 1e-30)
    assert err.max() <= REL_TOL, err.max()
    assert np.all(Y[g.nrows:] == 0)
    A.close()


def test_batch512_spmm_sampled_rows_against_fp64(pkg, cuda):
    """The uneven-batch configuration at full size: 512 Erdos-Renyi graphs (n
    log-uniform in 64..65536, degree U[4, 32]) stacked block-diagonally, FP32 X
    of width 64, the SpMM replayed from a captured CUDA graph.  A bounded sample
    of 4096 rows (every graph's first row among them) is checked against the
    FP64 product."""
    g, offsets, sizes, degrees = pkg.er_batch(512, 64, 65536, 4, 32, align=32, seed=4)
    k = 64
    X = np.random.default_rng(7).standard_normal((g.ncols, k)).astype(np.float32)
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    Xt = torch.from_numpy(X).to(cuda)
    Y = torch.empty(A.padded_rows(), k, device=cuda)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        A.spmm(Xt, Y)
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        A.spmm(Xt, Y)
    Y.zero_()
    graph.replay()
    torch.cuda.synchronize()
    Yn = Y.cpu().numpy()
    rng = np.random.default_rng(11)
    sample = np.unique(np.concatenate([offsets[:-1], rng.integers(0, g.nrows, 4096 - 512)]))
    X64 = X.astype(np.float64)
    for r in sample:
        cols = g.colind[g.rowptr[r]:g.rowptr[r + 1]]
        want = X64[cols].sum(0)
        scale = np.abs(X64[cols]).sum(0)
        err = np.abs(Yn[r] - want) / np.maximum(scale, 1e-30)
        assert err.max(initial=0.0) <= REL_TOL, (int(r), float(err.max()))
    A.close()
