"""The autotuner through the C ABI: it returns a packed matrix at one of the
candidate tile sizes with the chosen launch option applied, the result
multiplies correctly, and a second call for the same shape is served from the
cache (and from the cache file)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_util import REL_TOL, full_full_error

pytestmark = pytest.mark.gpu


def test_autotune_single_vector_and_cache(pkg, orc, cuda, tmp_path, monkeypatch):
    lib = pkg._lib.load()
    lib.b2sr_autotune_clear_cache()
    g = pkg.rmat(12, 16, seed=31)
    A, info = pkg.B2SRMatrix.autotuned(g, "bin_full_full", tile_dims=(4, 8, 16), device=cuda)
    assert info["tile_dim"] in (4, 8, 16) and A.tile_dim == info["tile_dim"]
    assert info["candidates"] >= 3 and info["best_ms"] > 0
    x = np.random.default_rng(1).random(g.ncols, dtype=np.float32)
    y = A.spmv_bin_full_full(torch.from_numpy(x).to(cuda)).cpu().numpy()
    assert full_full_error(orc, g, x, y) <= REL_TOL
    A2, info2 = pkg.B2SRMatrix.autotuned(g, "bin_full_full", tile_dims=(4, 8, 16), device=cuda)
    assert info2["candidates"] == 0 and info2["tile_dim"] == info["tile_dim"]
    assert A2.get_launch("bin_full_full")[3] == A.get_launch("bin_full_full")[3]
    A.close()
    A2.close()


def test_autotune_spmm_and_bits(pkg, orc, cuda):
    g = pkg.erdos_renyi(3000, 12.0, seed=5)
    A, info = pkg.B2SRMatrix.autotuned(g, "bin_full_full", k=64, device=cuda)
    X = torch.randn(g.ncols, 64, device=cuda)
    Y = A.spmm(X)
    dense = torch.zeros(g.nrows, g.ncols, device=cuda)
    dense[torch.from_numpy(np.repeat(np.arange(g.nrows), np.diff(g.rowptr))).to(cuda),
          torch.from_numpy(g.colind.astype(np.int64)).to(cuda)] = 1
    torch.testing.assert_close(Y[: g.nrows], dense @ X, rtol=1e-4, atol=1e-4)
    assert info["rhs_block"] in (0, 16, 32) and info["candidates"] >= 3  # k = 64: blocks 64, 32, 16
    B, binfo = pkg.B2SRMatrix.autotuned(g, "bin_bin_bin", device=cuda)
    assert binfo["algorithm"] in (1, 2)  # merge path or row-binned bit kernel, whichever timed faster
    xb = (np.random.default_rng(2).random(g.ncols) < 0.2).astype(np.float32)
    bits = B.spmv_bin_bin_bin(B.pack_bits(torch.from_numpy(xb).to(cuda)))
    got = B.unpack_bits(bits, g.nrows).cpu().numpy()
    want = (orc.csr_spmv_count(g.rowptr, g.colind, g.nrows, xb) > 0).astype(np.float32)
    np.testing.assert_array_equal(got, want)
