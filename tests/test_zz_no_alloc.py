"""The allocation-free multiply (b2sr_spmv_bin_full_full_noalloc), for callers
that cannot allocate device memory while they multiply, checked through the
C ABI against the allocating entry point b2sr_ref_bmv_bin_full_full on the
same B2SR arrays, two accumulating calls in a row.  Collected last so that a
run stopping at the first failure has run every other test before it."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from gpu_util import REL_TOL

pytestmark = pytest.mark.gpu


def _dev(a, cuda):
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_noalloc_matches_allocating_entry_point(pkg, cuda, T):
    lib = pkg._lib.load()
    g = pkg.rmat(13, 16, seed=21)
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    rp, ci, tl = A.download()
    nb = A.nblockrows
    d_rp = _dev(rp, cuda)
    d_ci = _dev(np.concatenate([ci, np.zeros(64, np.int32)]), cuda)
    d_tl = _dev(tl.view({4: np.uint8, 8: np.uint8, 16: np.int16, 32: np.int32}[T]), cuda)
    x_np = np.zeros(nb * T, np.float32)
    x_np[: g.ncols] = np.random.default_rng(T).standard_normal(g.ncols).astype(np.float32)
    x = _dev(x_np, cuda)
    y_alloc = torch.zeros(nb * T, device=cuda)
    y_free = torch.zeros(nb * T, device=cuda)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    scale = np.zeros(nb * T)
    rows = np.repeat(np.arange(g.nrows), np.diff(g.rowptr))
    np.add.at(scale, rows, np.abs(x_np[g.colind]).astype(np.float64))
    for call in range(2):
        torch.cuda.synchronize()
        rc = lib.b2sr_ref_bmv_bin_full_full(T, d_tl.data_ptr(), x.data_ptr(), y_alloc.data_ptr(), d_rp.data_ptr(),
                                            d_ci.data_ptr(), nb)
        assert rc == 0
        torch.cuda.synchronize()
        rc = lib.b2sr_spmv_bin_full_full_noalloc(T, d_tl.data_ptr(), d_rp.data_ptr(), d_ci.data_ptr(), nb, g.ncols,
                                                 x.data_ptr(), y_free.data_ptr(), 1, stream)
        assert rc == 0, pkg._lib.status_string(rc)
        torch.cuda.synchronize()
        a, b = y_alloc.cpu().numpy(), y_free.cpu().numpy()
        err = np.abs(a.astype(np.float64) - b) / np.maximum((call + 1) * scale, 1e-30)
        assert err.max() <= REL_TOL, f"T={T} call {call}: rel err {err.max():.3e}"
    A.close()


def test_noalloc_rejects_bad_arguments(pkg, cuda):
    lib = pkg._lib.load()
    y = torch.zeros(16, device=cuda)
    assert lib.b2sr_spmv_bin_full_full_noalloc(5, None, None, None, 4, 16, None, y.data_ptr(), 0, None) == 1
    assert lib.b2sr_spmv_bin_full_full_noalloc(4, None, None, None, 4, 16, None, None, 0, None) == 1
    assert lib.b2sr_spmv_bin_full_full_noalloc(4, None, None, None, 4, 16, y.data_ptr() + 4, y.data_ptr(), 0,
                                               None) == 1
