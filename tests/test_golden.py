"""Pins the oracle to the reference: outputs of the reference's own kernels
(tests/golden/*.npz, made by tests/golden/make_golden.py on a GPU from the
reference's bsrbmv.cu) must equal the oracle's on the same inputs.  CPU only."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
FILES = sorted(GOLDEN.glob("ref_*.npz"))


def test_fixtures_present():
    assert len(FILES) == 8, "expected rmat + uniform fixtures for T = 4, 8, 16, 32"


@pytest.mark.parametrize("path", FILES, ids=[p.stem for p in FILES])
def test_oracle_matches_reference_kernels(orc, path):
    f = np.load(path)
    T = int(f["T"])
    nrows = int(f["nrows"])
    rp, ci = f["csr_rowptr"], f["csr_colind"]
    # packing: ToBit{T}Col of cuSPARSE-order dense tiles == oracle layout
    brp, bci, tiles = orc.csr_to_b2sr(rp, ci, nrows, T)
    np.testing.assert_array_equal(brp, f["b2sr_rowptr"])
    np.testing.assert_array_equal(bci, f["b2sr_colind"])
    np.testing.assert_array_equal(tiles, f["ref_tiles"])
    # vector bits: ToBit{T}Row
    xbits = orc.pack_vec_bits(f["xbool"], T)
    np.testing.assert_array_equal(xbits, f["ref_xbits"])
    # multiplies
    np.testing.assert_array_equal(orc.bmv_bin_bin_bin(T, brp, bci, tiles, xbits), f["ref_y_bbb"])
    np.testing.assert_array_equal(orc.bmv_bin_bin_full(T, brp, bci, tiles, xbits), f["ref_y_bbf"])
    if "ref_y_bff" in f.files:
        y = orc.bmv_bin_full_full(T, brp, bci, tiles, f["x"])
        ref = f["ref_y_bff"]
        if T == 32:
            # bmv32_bin_full_full sums in the oracle's order: bit-exact
            np.testing.assert_array_equal(y, ref)
        else:
            # T < 32 reference kernels add lane partials with atomicAdd
            np.testing.assert_allclose(y, ref, rtol=1e-6, atol=1e-6)
        y64 = orc.csr_spmv_f64(rp, ci, nrows, f["x"])
        np.testing.assert_allclose(ref[:nrows], y64, rtol=1e-5)
