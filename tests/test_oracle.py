"""CPU tests of the oracle: hand-derived known answers in the reference's bit
layout, and agreement between the oracle's B2SR path and its independent CSR
path.  (The reference ships no golden vectors; tests/golden/ holds outputs of
the reference's own kernels, checked in test_golden.py.)"""
from __future__ import annotations

import numpy as np
import pytest


def csr_from_dense(d):
    d = np.asarray(d)
    rp = [0]
    ci = []
    for row in d:
        nz = np.nonzero(row)[0]
        ci.extend(nz.tolist())
        rp.append(len(ci))
    return np.array(rp, np.int32), np.array(ci, np.int32)


# A 4x4 matrix; rows as bit strings (column 0 first).
DENSE4 = [[1, 0, 0, 1],
          [0, 1, 0, 0],
          [0, 0, 1, 0],
          [1, 0, 0, 0]]


def test_tile_layout_t4(orc):
    # ToBit4Col (bmv_eval/backend/bsrbmv.cu:33-62): one byte per tile row, low
    # nibble, column c at bit 3-c.
    rp, ci = csr_from_dense(DENSE4)
    brp, bci, tiles = orc.csr_to_b2sr(rp, ci, 4, 4)
    assert brp.tolist() == [0, 1]
    assert bci.tolist() == [0]
    assert tiles.tolist() == [0b1001, 0b0100, 0b0010, 0b1000]


def test_tile_layout_t8_two_tiles(orc):
    d = np.zeros((8, 16), np.int8)
    d[0, [0, 7, 8, 15]] = 1
    d[5, 9] = 1
    rp, ci = csr_from_dense(d)
    brp, bci, tiles = orc.csr_to_b2sr(rp, ci, 8, 8)
    assert brp.tolist() == [0, 2]
    assert bci.tolist() == [0, 1]
    assert tiles.tolist() == [0x81, 0, 0, 0, 0, 0, 0, 0,
                              0x81, 0, 0, 0, 0, 0x40, 0, 0]


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_tile_layout_msb_is_column_zero(orc, T):
    # entry (r, c) of tile (0, 1) sets bit T-1-c of word r
    for r, c in [(0, 0), (T - 1, T - 1), (1, T - 2)]:
        rp = np.zeros(T + 1, np.int32)
        rp[r + 1:] = 1
        ci = np.array([T + c], np.int32)
        brp, bci, tiles = orc.csr_to_b2sr(rp, ci, T, T)
        assert bci.tolist() == [1]
        want = np.zeros(T, np.uint64)
        want[r] = 1 << (T - 1 - c)
        assert tiles.astype(np.uint64).tolist() == want.tolist()


def test_ragged_rows_and_empty_tilerows(orc):
    # 9 rows with T = 4: tile-row 2 holds only row 8; tile-row 1 is empty.
    d = np.zeros((9, 9), np.int8)
    d[0, 8] = 1
    d[8, 0] = 1
    d[8, 5] = 1
    rp, ci = csr_from_dense(d)
    brp, bci, tiles = orc.csr_to_b2sr(rp, ci, 9, 4)
    assert brp.tolist() == [0, 1, 1, 3]
    assert bci.tolist() == [2, 0, 1]
    assert tiles.tolist() == [0b1000, 0, 0, 0,    # (0, 8): row 0, col 0 of tile-col 2
                              0b1000, 0, 0, 0,    # (8, 0)
                              0b0100, 0, 0, 0]    # (8, 5): col 1 of tile-col 1


def test_vector_bits_known_answers(orc):
    # ToBit4Row (bmv_eval/backend/bsrbmv.cu:64-90): x[4k] at bit 3 of byte k.
    x = np.array([1, 0, 0, 1, 0, 1, 1, 0, 0.5], np.float32)
    assert orc.pack_vec_bits(x, 4).tolist() == [0b1001, 0b0110, 0b1000]
    assert orc.pack_vec_bits(x, 8).tolist() == [0b10010110, 0b10000000]
    b32 = orc.pack_vec_bits(x, 32)
    assert b32.tolist() == [0b10010110_1 << 23]
    # x > 0 is the test, as in ToBit{T}Row: negatives and zeros give 0
    assert orc.pack_vec_bits(np.array([-1, 0, 2, -0.0], np.float32), 4).tolist() == [0b0010]
    np.testing.assert_array_equal(orc.unpack_vec_bits(orc.pack_vec_bits(x, 8), 9, 8), (x > 0).astype(np.float32))


def test_multiply_known_answers_t4(orc):
    rp, ci = csr_from_dense(DENSE4)
    brp, bci, tiles = orc.csr_to_b2sr(rp, ci, 4, 4)
    xb = np.array([0b1100], np.uint8)  # x0 = x1 = 1
    assert orc.bmv_bin_bin_full(4, brp, bci, tiles, xb).tolist() == [1, 1, 0, 1]
    assert orc.bmv_bin_bin_count(4, brp, bci, tiles, xb).tolist() == [1, 1, 0, 1]
    assert orc.bmv_bin_bin_bin(4, brp, bci, tiles, xb).tolist() == [0b1101]
    x = np.array([1, 2, 4, 8], np.float32)
    assert orc.bmv_bin_full_full(4, brp, bci, tiles, x).tolist() == [9, 2, 4, 1]
    # accumulate adds (full) / ORs (bits), as the reference kernels do
    y0 = np.array([1, 1, 1, 1], np.float32)
    assert orc.bmv_bin_full_full(4, brp, bci, tiles, x, y0, True).tolist() == [10, 3, 5, 2]
    assert orc.bmv_bin_bin_bin(4, brp, bci, tiles, xb, np.array([0b0010], np.uint8), True).tolist() == [0b1111]
    # masked BFS step: visited rows 0 and 3 are cleared
    assert orc.bmv_bin_bin_bin_masked(4, brp, bci, tiles, xb, np.array([0b1001], np.uint8)).tolist() == [0b0100]


def _random_graphs(pkg):
    yield pkg.erdos_renyi(300, 6.0, seed=3)
    yield pkg.rmat(9, 8, seed=5)
    yield pkg.from_edges([0, 0, 2, 7, 7, 7], [1, 6, 2, 0, 3, 6], nrows=11, ncols=13)


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_b2sr_path_agrees_with_csr_path(pkg, orc, T):
    rng = np.random.default_rng(T)
    for g in _random_graphs(pkg):
        brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
        nb = (g.nrows + T - 1) // T
        assert len(brp) == nb + 1 and brp[-1] == len(bci)
        # every set bit is one CSR entry
        assert int(sum(bin(int(w)).count("1") for w in tiles)) == g.nnz
        x = np.zeros(max(nb, (g.ncols + T - 1) // T) * T, np.float32)
        x[: g.ncols] = rng.random(g.ncols, dtype=np.float32)
        y64 = orc.bmv_bin_full_full_f64(T, brp, bci, tiles, x)[: g.nrows]
        np.testing.assert_allclose(y64, orc.csr_spmv_f64(g.rowptr, g.colind, g.nrows, x), rtol=1e-12)
        y32 = orc.bmv_bin_full_full(T, brp, bci, tiles, x)[: g.nrows]
        np.testing.assert_allclose(y32, y64, rtol=1e-5)
        xbool = np.zeros_like(x)
        xbool[: g.ncols] = rng.random(g.ncols) < 0.3
        xb = orc.pack_vec_bits(xbool, T)
        cnt = orc.csr_spmv_count(g.rowptr, g.colind, g.nrows, xbool)
        assert orc.bmv_bin_bin_count(T, brp, bci, tiles, xb)[: g.nrows].tolist() == cnt.tolist()
        assert orc.bmv_bin_bin_full(T, brp, bci, tiles, xb)[: g.nrows].tolist() == cnt.astype(np.float32).tolist()
        ybits = orc.bmv_bin_bin_bin(T, brp, bci, tiles, xb)
        assert orc.unpack_vec_bits(ybits, g.nrows, T).tolist() == (cnt > 0).astype(np.float32).tolist()


def test_cpu_baseline_matches_oracle(pkg, orc):
    g = pkg.rmat(10, 16, seed=2)
    x = np.random.default_rng(0).random(g.ncols, dtype=np.float32)
    y, used = orc.csr_spmv_f32_omp(g.rowptr, g.colind, g.nrows, x)
    assert used >= 1
    np.testing.assert_allclose(y, orc.csr_spmv_f64(g.rowptr, g.colind, g.nrows, x), rtol=1e-5)


@pytest.mark.parametrize("scale", [6, 12])
def test_oracle_rmat_builds_the_library_graph(pkg, orc, scale):
    # the benchmark's CPU arm builds its input with the oracle alone; it must
    # be the library's graph bit for bit
    rp, ci = orc.rmat_csr(scale, 16, 0.57, 0.19, 0.19, 1)
    g = pkg.rmat(scale, 16, 0.57, 0.19, 0.19, 1)
    assert np.array_equal(rp, g.rowptr) and np.array_equal(ci, g.colind)


def test_oracle_sym_csr_canonical_form(orc):
    u = np.array([0, 2, 2, 1, 3, 3, 0], np.int32)
    v = np.array([1, 0, 0, 1, 2, 0, 1], np.int32)  # duplicate, self-loop, both directions
    rowptr = np.empty(5, np.int32)
    colind = np.empty(2 * u.size, np.int32)
    nnz = orc._load().oracle_sym_csr(u.ctypes.data, v.ctypes.data, u.size, 4, rowptr.ctypes.data,
                                     colind.ctypes.data)
    assert nnz == 8
    assert rowptr.tolist() == [0, 3, 4, 6, 8]
    assert colind[:nnz].tolist() == [1, 2, 3, 0, 0, 3, 0, 2]
