"""Speed against the reference's own kernels on the same GPU and the same
device buffers (the reference's bsrbmv.cu compiled for sm_103a, oracle/_ref/):
the bit-vector variants on the R-MAT scale-20 graph of the benchmark, and
bin_full_full on a uniform-load matrix with the same tile count (the reference
bin_full_full kernels are defined only for equal tiles per tile-row; see
ref_kernels).  Results must match; our kernels must be faster.  Run with -s to
see the table."""
from __future__ import annotations

import statistics

import numpy as np
import pytest
import torch

import ref_kernels as rk
from gpu_util import to_np_words

pytestmark = pytest.mark.gpu

WORD = {4: torch.uint8, 8: torch.uint8, 16: torch.int16, 32: torch.int32}
NPW = {4: np.uint8, 8: np.uint8, 16: np.int16, 32: np.int32}


@pytest.fixture(scope="module")
def ref(cuda):
    if not rk.available():
        pytest.fail("reference cubin missing: oracle/_ref/ was not built from the reference checkout")
    return rk.RefKernels()


@pytest.fixture(scope="module")
def flush(cuda):
    return torch.ones(64 << 20, device=cuda)


def median_us(fn, flush, reps=15):
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    evs = []
    for _ in range(reps):
        flush.amax()  # read-only L2 eviction between launches
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        evs.append((a, b))
    torch.cuda.synchronize()
    return statistics.median(a.elapsed_time(b) for a, b in evs) * 1e3


@pytest.fixture(scope="module")
def rmat20(pkg):
    return pkg.rmat(20, 16, 0.57, 0.19, 0.19, 1)


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_bit_variants_faster_than_reference(pkg, ref, cuda, flush, rmat20, T):
    g = rmat20
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    nb = A.nblockrows
    rk.check_bits_input(T, nb)
    brp, bci, tiles = A.download()
    d_rp = torch.from_numpy(brp).to(cuda)
    d_ci = torch.zeros(len(bci) + 64, dtype=torch.int32, device=cuda)
    d_ci[: len(bci)] = torch.from_numpy(bci).to(cuda)
    d_tl = torch.from_numpy(tiles.view(NPW[T])).to(cuda)
    frontier = (torch.from_numpy(np.random.default_rng(3).random(g.ncols)).to(cuda) < 0.01).float()
    xb = torch.zeros(rk.xbits_len(nb, T), dtype=WORD[T], device=cuda)
    xb[: A.nblockcols] = A.pack_bits(frontier)
    yr = torch.zeros(nb + 64, dtype=WORD[T], device=cuda)
    yf = torch.zeros(nb * T + 64, device=cuda)
    yo = torch.empty(nb, dtype=WORD[T], device=cuda)
    yc = torch.empty(nb * T, device=cuda)
    t = {
        "ref bin_bin_bin": median_us(lambda: ref.bmv("bin_bin_bin", T, d_tl, xb, yr, d_rp, d_ci, nb), flush),
        "ref bin_bin_full": median_us(lambda: ref.bmv("bin_bin_full", T, d_tl, xb, yf, d_rp, d_ci, nb), flush),
        "ours bin_bin_bin": median_us(lambda: A.spmv_bin_bin_bin(xb, yo), flush),
        "ours bin_bin_full": median_us(lambda: A.spmv_bin_bin_full(xb, yc), flush),
    }
    yr.zero_()
    ref.bmv("bin_bin_bin", T, d_tl, xb, yr, d_rp, d_ci, nb)
    yf.zero_()
    ref.bmv("bin_bin_full", T, d_tl, xb, yf, d_rp, d_ci, nb)
    np.testing.assert_array_equal(to_np_words(yr, T)[:nb], to_np_words(A.spmv_bin_bin_bin(xb), T))
    assert torch.equal(yf[: nb * T], A.spmv_bin_bin_full(xb))
    print(f"\nR-MAT s20 T={T}: " + ", ".join(f"{k} {v:.1f} us" for k, v in t.items()))
    assert t["ours bin_bin_bin"] < t["ref bin_bin_bin"]
    assert t["ours bin_bin_full"] < t["ref bin_bin_full"]
    A.close()


@pytest.mark.parametrize("T,nb,per_row", [(4, 262144, 104), (8, 131072, 181), (32, 32768, 225)])
def test_full_full_faster_than_reference(pkg, ref, cuda, flush, T, nb, per_row):
    rng = np.random.default_rng(T)
    stride = nb // per_row  # distinct ascending tile-columns per tile-row
    bci = (np.arange(per_row)[None, :] * stride + rng.integers(0, stride, (nb, per_row))).astype(np.int32).ravel()
    brp = (np.arange(nb + 1, dtype=np.int64) * per_row).astype(np.int32)
    nt = len(bci)
    pos = rng.integers(0, T * T, nt)  # one set bit per tile (R-MAT averages 1.15 at T = 4)
    wdt = {4: np.uint8, 8: np.uint8, 16: np.uint16, 32: np.uint32}[T]
    words = np.zeros((nt, T), wdt)
    words[np.arange(nt), pos // T] = (np.uint64(1) << (np.uint64(T - 1) - (pos % T).astype(np.uint64))).astype(wdt)
    tiles = np.concatenate([words.ravel(), np.zeros(64 * T, wdt)])
    d_rp = torch.from_numpy(brp).to(cuda)
    d_ci = torch.zeros(nt + 64, dtype=torch.int32, device=cuda)
    d_ci[:nt] = torch.from_numpy(bci).to(cuda)
    d_tl = torch.from_numpy(tiles.view(NPW[T])).to(cuda)
    rk.check_full_full_input(brp)
    A = pkg.B2SRMatrix.wrap(d_rp, d_ci[:nt], d_tl, nb * T, nb * T, T)
    x = torch.rand(rk.x_float_len(nb, T), device=cuda)
    yr = torch.zeros(nb * T + 64, device=cuda)
    yo = torch.empty(nb * T, device=cuda)
    t_ref = median_us(lambda: ref.bmv("bin_full_full", T, d_tl, x, yr, d_rp, d_ci, nb), flush)
    t_ours = median_us(lambda: A.spmv_bin_full_full(x, yo), flush)
    yr.zero_()
    ref.bmv("bin_full_full", T, d_tl, x, yr, d_rp, d_ci, nb)
    y = A.spmv_bin_full_full(x)
    torch.testing.assert_close(y, yr[: nb * T], rtol=2e-6, atol=1e-6)
    print(f"\nuniform nb={nb} T={T} tiles={nt}: ref bin_full_full {t_ref:.1f} us, ours {t_ours:.1f} us")
    assert t_ours < t_ref
    A.close()
