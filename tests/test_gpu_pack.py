"""GPU parity of the device packer and the vector bit conversion against the
oracle (bit-exact), through the C ABI."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from gpu_util import from_np_words, graph_zoo, to_np_words

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def zoo(pkg):
    return graph_zoo(pkg)


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_pack_bit_exact(pkg, orc, cuda, zoo, T):
    for name, g in zoo.items():
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        brp, bci, tiles = A.download()
        wrp, wci, wtiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
        assert A.nblockrows == (g.nrows + T - 1) // T, name
        assert A.nblocks == len(wci), name
        assert A.nnz == g.nnz, name
        np.testing.assert_array_equal(brp, wrp, err_msg=name)
        np.testing.assert_array_equal(bci, wci, err_msg=name)
        np.testing.assert_array_equal(tiles, wtiles, err_msg=name)
        A.close()


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_transpose_bit_exact(pkg, orc, cuda, zoo, T):
    for name in ("rect_70x333", "rmat_s12", "hub_40000", "single_row"):
        g = zoo[name]
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        At = A.transpose()
        rows = np.repeat(np.arange(g.nrows), np.diff(g.rowptr))
        gt = pkg.from_edges(g.colind, rows, nrows=g.ncols, ncols=g.nrows, drop_self_loops=False)
        wrp, wci, wtiles = orc.csr_to_b2sr(gt.rowptr, gt.colind, gt.nrows, T)
        brp, bci, tiles = At.download()
        assert (At.nrows, At.ncols) == (g.ncols, g.nrows)
        np.testing.assert_array_equal(brp, wrp, err_msg=name)
        np.testing.assert_array_equal(bci, wci, err_msg=name)
        np.testing.assert_array_equal(tiles, wtiles, err_msg=name)
        A.close()



@pytest.mark.parametrize("T", [4, 32])
def test_transpose_three_digit_passes(pkg, orc, cuda, T):
    """A 5,000 x 300,000 graph with a quarter of its edges on 8 hub columns:
    at T = 4 its 75,000 tile-columns take three 8-bit digit passes of the
    device sort (two at T = 32).  The transposed B2SR equals the oracle's
    packing of the transposed CSR, so the sort kept tile-row order inside
    every tile-column."""
    rng = np.random.default_rng(21)
    nrows, ncols, ne = 5000, 300000, 400000
    rows = rng.integers(0, nrows, ne)
    cols = rng.integers(0, ncols, ne)
    cols[: ne // 4] = rng.integers(0, 8, ne // 4)
    g = pkg.from_edges(rows, cols, nrows=nrows, ncols=ncols, drop_self_loops=False)
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    At = A.transpose()
    rr = np.repeat(np.arange(g.nrows), np.diff(g.rowptr))
    gt = pkg.from_edges(g.colind, rr, nrows=g.ncols, ncols=g.nrows, drop_self_loops=False)
    wrp, wci, wtiles = orc.csr_to_b2sr(gt.rowptr, gt.colind, gt.nrows, T)
    brp, bci, tiles = At.download()
    assert (At.nrows, At.ncols, At.nnz) == (g.ncols, g.nrows, g.nnz)
    np.testing.assert_array_equal(brp, wrp)
    np.testing.assert_array_equal(bci, wci)
    np.testing.assert_array_equal(tiles, wtiles)
    A.close()


def test_transpose_rejects_tile_column_out_of_range(pkg, cuda):
    """Wrapped arrays whose tile-column lies past the last one: the transpose
    reports B2SR_ERR_INVALID_VALUE (its kernels only sort and copy the column
    values; no multiply runs)."""
    rowptr = torch.tensor([0, 1], dtype=torch.int32, device=cuda)
    colind = torch.tensor([5], dtype=torch.int32, device=cuda)
    tiles = torch.tensor([8, 0, 0, 0], dtype=torch.uint8, device=cuda)
    A = pkg.B2SRMatrix.wrap(rowptr, colind, tiles, 4, 4, 4)
    with pytest.raises(pkg.B2SRError) as e:
        A.transpose()
    assert e.value.status == 1
    A.close()

def test_invalid_csr_is_rejected_without_packing(pkg, cuda):
    lib = pkg._lib.load()
    out = C.c_void_p()
    cases = {
        "descending rowptr": ([0, 3, 2, 4], [0, 1, 2, 3]),
        "column out of range": ([0, 1, 2, 3], [0, 1, 9]),
        "unsorted row": ([0, 3, 3, 3], [2, 0, 1]),
        "rowptr[n] != nnz": ([0, 1, 2, 2], [0, 1, 2]),
        "negative column": ([0, 1, 1, 1], [-1]),
    }
    for what, (rp, ci) in cases.items():
        rpt = torch.tensor(rp, dtype=torch.int32, device=cuda)
        cit = torch.tensor(ci, dtype=torch.int32, device=cuda)
        rc = lib.b2sr_pack_csr(rpt.data_ptr(), cit.data_ptr(), 3, 4, len(ci), 4, None, C.byref(out))
        assert rc == 2, what
        assert out.value is None
    # the context is still usable
    torch.cuda.synchronize()
    with pytest.raises(pkg.B2SRError):
        pkg.B2SRMatrix.from_csr(np.array([0, 2, 1]), np.array([1, 0]), 2, 2, 8, device=cuda)


def test_duplicates_in_csr_merge(pkg, orc, cuda):
    rp = np.array([0, 3, 4], np.int32)
    ci = np.array([1, 1, 5, 5], np.int32)
    A = pkg.B2SRMatrix.from_csr(rp, ci, 2, 8, 4, device=cuda)
    assert A.nnz == 3
    brp, bci, tiles = A.download()
    assert bci.tolist() == [0, 1] and tiles.tolist() == [0b0100, 0, 0, 0, 0b0100, 0b0100, 0, 0]


@pytest.mark.parametrize("T", [4, 8, 16, 32])
@pytest.mark.parametrize("n", [1, 5, 31, 32, 33, 100, 4097, 1 << 20])
def test_vector_bits_round_trip(pkg, orc, cuda, T, n):
    rng = np.random.default_rng(n + T)
    x = (rng.random(n) - 0.3).astype(np.float32)
    x[rng.random(n) < 0.1] = 0.0
    bits = pkg.pack_vec_bits(torch.from_numpy(x).to(cuda), T)
    want = orc.pack_vec_bits(x, T)
    np.testing.assert_array_equal(to_np_words(bits, T), want)
    back = pkg.unpack_vec_bits(from_np_words(want, T, cuda), T, n)
    np.testing.assert_array_equal(back.cpu().numpy(), orc.unpack_vec_bits(want, n, T))


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_packed_file_round_trip_and_checks(pkg, cuda, tmp_path, T):
    """save -> load gives the same arrays and products; a flipped payload byte,
    a truncated file and a wrong magic are refused with B2SR_ERR_IO (8)."""
    g = pkg.rmat(11, 8, seed=T)
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    path = tmp_path / f"m{T}.b2sr"
    A.save(path)
    B = pkg.B2SRMatrix.load(path, device=cuda)
    for a, b in zip(A.download(), B.download()):
        np.testing.assert_array_equal(a, b)
    assert (B.nrows, B.ncols, B.nnz, B.tile_dim) == (A.nrows, A.ncols, A.nnz, A.tile_dim)
    x = torch.rand(g.ncols, device=cuda)
    assert torch.equal(A.spmv_bin_full_full(x), B.spmv_bin_full_full(x))
    data = bytearray(path.read_bytes())
    for name, bad in (("flip", data[:100] + bytes([data[100] ^ 1]) + data[101:]),
                      ("short", data[:-5]),
                      ("magic", b"X" + data[1:])):
        p2 = tmp_path / f"{name}{T}.b2sr"
        p2.write_bytes(bytes(bad))
        with pytest.raises(pkg.B2SRError) as ei:
            pkg.B2SRMatrix.load(p2, device=cuda)
        assert ei.value.status == 8, name
    with pytest.raises(pkg.B2SRError):
        pkg.B2SRMatrix.load(tmp_path / "missing.b2sr", device=cuda)
    A.close()
    B.close()


@pytest.mark.parametrize("T", [4, 32])
def test_zero_size_matrices(pkg, cuda, tmp_path, T):
    """0 x 0 and 0 x n matrices pack, multiply (all variants), transpose and
    round-trip through a file without touching memory they do not own."""
    for nrows, ncols in ((0, 0), (0, 50), (50, 0)):
        g = pkg.from_edges([], [], nrows=nrows, ncols=ncols)
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        assert (A.nblocks, A.nnz) == (0, 0)
        x = torch.ones(max(ncols, 1), device=cuda)
        y = A.spmv_bin_full_full(x)
        assert y.numel() >= A.padded_rows() and bool(torch.all(y[: A.padded_rows()] == 0))
        xb = A.pack_bits(x[: max(ncols, 1)], max(ncols, 0) or 1)
        assert bool(torch.all(A.spmv_bin_bin_count(xb)[: A.padded_rows()] == 0))
        Y = A.spmm(torch.ones(max(ncols, 1), 8, device=cuda))
        assert bool(torch.all(Y[: A.padded_rows()] == 0))
        Ym = A.spmv_multi_bits(torch.ones(max(ncols, 1), dtype=torch.int64, device=cuda))
        assert bool(torch.all(Ym[: A.padded_rows()] == 0))
        At = A.transpose()
        assert (At.nrows, At.ncols, At.nblocks) == (ncols, nrows, 0)
        path = tmp_path / f"z{nrows}_{ncols}_{T}.b2sr"
        A.save(path)
        B = pkg.B2SRMatrix.load(path, device=cuda)
        assert (B.nrows, B.ncols, B.nblocks) == (nrows, ncols, 0)
        B.close()
        A.close()
