"""The allocation-free multiply (b2sr_spmv_bin_full_full_noalloc), for callers
that cannot allocate device memory while they multiply, checked through the
C ABI: two accumulating calls in a row against the allocating entry point
b2sr_ref_bmv_bin_full_full on the same B2SR arrays (a different kernel: the
shim runs the row-binned plan, the no-alloc call the merge path) and against
the FP64 CSR oracle, with a counting allocator installed to show that the
calls allocate nothing.  Collected last so that a run stopping at the first
failure has run every other test before it."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from gpu_util import REL_TOL

pytestmark = pytest.mark.gpu


def _dev(a, cuda):
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


class CountingAllocator:
    """Installs b2sr_set_allocator hooks that count the library's device
    allocations and serve none (every request would fail), restoring the
    default allocator on exit."""

    def __init__(self, L):
        self.L = L
        self.allocs = 0
        self.frees = 0

        def alloc(nbytes, ctx):
            self.allocs += 1
            return None

        def free(ptr, ctx):
            self.frees += 1

        self._alloc = L.ALLOC_FN(alloc)  # referenced while installed
        self._free = L.FREE_FN(free)

    def __enter__(self):
        self.L.load().b2sr_set_allocator(self._alloc, self._free, None)
        return self

    def __exit__(self, *exc):
        self.L.load().b2sr_set_allocator(self.L.ALLOC_FN(), self.L.FREE_FN(), None)


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_noalloc_matches_allocating_entry_point_and_fp64(pkg, orc, cuda, T):
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
    y64 = orc.csr_spmv_f64(g.rowptr, g.colind, g.nrows, x_np[: g.ncols])
    scale = np.maximum(orc.csr_spmv_abs_f64(g.rowptr, g.colind, g.nrows, x_np[: g.ncols]), 1e-30)
    try:
        _two_calls(pkg, lib, T, g, nb, d_tl, d_rp, d_ci, x, y_alloc, y_free, stream, y64, scale)
    finally:
        lib.b2sr_ref_release(None)  # the shim caches a plan of these arrays, freed with this test
    A.close()


def _two_calls(pkg, lib, T, g, nb, d_tl, d_rp, d_ci, x, y_alloc, y_free, stream, y64, scale):
    for call in range(2):
        torch.cuda.synchronize()
        rc = lib.b2sr_ref_bmv_bin_full_full(T, d_tl.data_ptr(), x.data_ptr(), y_alloc.data_ptr(), d_rp.data_ptr(),
                                            d_ci.data_ptr(), nb)
        assert rc == 0
        torch.cuda.synchronize()
        with CountingAllocator(pkg._lib) as counter:
            rc = lib.b2sr_spmv_bin_full_full_noalloc(T, d_tl.data_ptr(), d_rp.data_ptr(), d_ci.data_ptr(), nb,
                                                     g.ncols, x.data_ptr(), y_free.data_ptr(), 1, stream)
            torch.cuda.synchronize()
        assert rc == 0, pkg._lib.status_string(rc)
        assert counter.allocs == 0 and counter.frees == 0, "the no-alloc call asked the library allocator"
        a, b = y_alloc.cpu().numpy(), y_free.cpu().numpy()
        k = call + 1  # accumulated calls so far
        err = np.abs(a.astype(np.float64) - b)[: g.nrows] / (k * scale)
        assert err.max() <= REL_TOL, f"T={T} call {call}: vs the allocating entry point {err.max():.3e}"
        err64 = np.abs(b[: g.nrows].astype(np.float64) - k * y64) / (k * scale)
        print(f"T={T} call {call}: max error vs FP64 {err64.max():.2e} (row-abs-sum scaled)")
        assert err64.max() <= REL_TOL, f"T={T} call {call}: vs FP64 {err64.max():.3e}"
        assert not np.any(b[g.nrows:]), "padding rows must stay zero"


def test_noalloc_rejects_bad_arguments(pkg, cuda):
    lib = pkg._lib.load()
    y = torch.zeros(16, device=cuda)
    x = torch.zeros(16, device=cuda)
    p = y.data_ptr()
    assert lib.b2sr_spmv_bin_full_full_noalloc(5, None, None, None, 4, 16, None, p, 0, None) == 1
    assert lib.b2sr_spmv_bin_full_full_noalloc(4, None, None, None, 4, 16, None, None, 0, None) == 1
    assert lib.b2sr_spmv_bin_full_full_noalloc(4, None, None, None, 4, 16, p + 4, p, 0, None) == 1
    # with rows to compute, a null x, tile or colind array is refused before any launch
    assert lib.b2sr_spmv_bin_full_full_noalloc(4, p, p, p, 4, 16, None, p, 0, None) == 1
    assert lib.b2sr_spmv_bin_full_full_noalloc(4, None, p, p, 4, 16, x.data_ptr(), p, 0, None) == 1
    assert lib.b2sr_spmv_bin_full_full_noalloc(4, p, p, None, 4, 16, x.data_ptr(), p, 0, None) == 1
    # no rows: nothing to do, nothing read
    assert lib.b2sr_spmv_bin_full_full_noalloc(4, None, p, None, 0, 0, None, p, 0, None) == 0
