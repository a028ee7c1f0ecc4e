"""Our CUDA path against the reference's own kernels on the same device buffers
(the reference's bsrbmv.cu compiled for sm_103a, oracle/_ref/): bit-exact for
bin_bin_bin and bin_bin_full, FP32 tolerance for bin_full_full, plus the
reference ToBit{T}Row/ToBit{T}Col packers against ours.  Inputs satisfy the
conditions under which the reference kernels are well defined (see ref_kernels)."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest
import torch

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import ref_kernels as rk  # noqa: E402
from make_golden import WORD_T, b2sr_structure_numpy, uniform_case  # noqa: E402

from gpu_util import to_np_words  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref(cuda):
    if not rk.available():
        pytest.fail("reference cubin missing: oracle/_ref/ was not built from the reference checkout")
    return rk.RefKernels()


def _pad_colind(bci, dev):
    d = torch.zeros(len(bci) + 64, dtype=torch.int32, device=dev)
    d[: len(bci)] = torch.from_numpy(np.ascontiguousarray(bci)).to(dev)
    return d


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_packers_match_reference(pkg, ref, cuda, T):
    g = pkg.rmat(11, 8, seed=T)
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    _, _, tiles = A.download()
    brp, bci, dense = b2sr_structure_numpy(g.rowptr, g.colind, g.nrows, T)
    d_tiles = torch.zeros(rk.packed_tiles_len(len(bci), T), dtype=WORD_T[T], device=cuda)
    ref.to_bit_col(T, torch.from_numpy(dense).to(cuda), d_tiles, len(bci))
    np.testing.assert_array_equal(to_np_words(d_tiles, T)[: len(bci) * T], tiles)
    nb = A.nblockrows
    x = np.zeros(rk.x_float_len(nb, T), np.float32)
    x[: g.ncols] = (np.random.default_rng(T).random(g.ncols) < 0.4)
    d_xb = torch.zeros(rk.xbits_len(nb, T), dtype=WORD_T[T], device=cuda)
    ref.to_bit_row(T, torch.from_numpy(x).to(cuda), d_xb, nb)
    ours = A.pack_bits(torch.from_numpy(x[: g.ncols]).to(cuda))
    np.testing.assert_array_equal(to_np_words(d_xb, T)[: A.nblockcols], to_np_words(ours, T))
    A.close()


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_bit_variants_match_reference(pkg, ref, cuda, T):
    g = pkg.rmat(12, 16, seed=10 + T)  # nblockrows a multiple of 8 for every T
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    nb = A.nblockrows
    rk.check_bits_input(T, nb)
    brp, bci, tiles = A.download()
    d_rp = torch.from_numpy(brp).to(cuda)
    d_ci = _pad_colind(bci, cuda)
    d_tiles = torch.from_numpy(tiles.view({4: np.uint8, 8: np.uint8, 16: np.int16, 32: np.int32}[T])).to(cuda)
    xb = A.pack_bits(torch.from_numpy((np.random.default_rng(1).random(g.ncols) < 0.3).astype(np.float32)).to(cuda))
    yr = torch.zeros(nb + 64, dtype=WORD_T[T], device=cuda)
    ref.bmv("bin_bin_bin", T, d_tiles, xb, yr, d_rp, d_ci, nb)
    ours = A.spmv_bin_bin_bin(xb)
    np.testing.assert_array_equal(to_np_words(yr, T)[:nb], to_np_words(ours, T))
    yf = torch.zeros(nb * T + 64, device=cuda)
    ref.bmv("bin_bin_full", T, d_tiles, xb, yf, d_rp, d_ci, nb)
    np.testing.assert_array_equal(yf[: nb * T].cpu().numpy(), A.spmv_bin_bin_full(xb).cpu().numpy())
    A.close()


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_full_full_matches_reference(pkg, ref, cuda, T):
    g = uniform_case(T, nb=128, per_row=9, seed=7)
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    brp, bci, tiles = A.download()
    rk.check_full_full_input(brp)
    nb = A.nblockrows
    x = np.random.default_rng(T).random(nb * T, dtype=np.float32)
    xd = torch.from_numpy(x).to(cuda)
    d_tiles = torch.from_numpy(tiles.view({4: np.uint8, 8: np.uint8, 16: np.int16, 32: np.int32}[T])).to(cuda)
    yr = torch.zeros(nb * T + 64, device=cuda)
    ref.bmv("bin_full_full", T, d_tiles, xd, yr, torch.from_numpy(brp).to(cuda), _pad_colind(bci, cuda), nb)
    ours = A.spmv_bin_full_full(xd).cpu().numpy()
    np.testing.assert_allclose(ours, yr[: nb * T].cpu().numpy(), rtol=2e-6, atol=1e-6)
    A.close()
