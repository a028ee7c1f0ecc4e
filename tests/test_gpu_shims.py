"""The reference-compatible shims as the reference drivers use them: pack
through b2sr_ref_csr2bsr_nnz / b2sr_ref_csr2bsr_batch into caller-owned
arrays, then launch b2sr_ref_bmv_* several times with accumulation
(bmv_eval/test_bin_full_full.cu:167-211, 285-297).  Checked against the
oracle; the cached plan must follow a re-pack into the same arrays; and on
R-MAT scale 20 a shim call must cost what the matrix API's call costs."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from gpu_util import REL_TOL, to_np_words

pytestmark = pytest.mark.gpu

WORD = {4: np.uint8, 8: np.uint8, 16: np.int16, 32: np.int32}


@pytest.fixture
def shim_lib(pkg):
    lib = pkg._lib.load()
    yield lib
    torch.cuda.synchronize()
    lib.b2sr_ref_release(None)  # cached plans of this test's arrays


def ref_pack(lib, g, T, cuda, nt_cap=None):
    """B2SR arrays packed by the shims into caller-owned tensors (the driver's CSR2HSBSF)."""
    nb = (g.nrows + T - 1) // T
    d_csr_rp = torch.from_numpy(g.rowptr).to(cuda)
    d_csr_ci = torch.from_numpy(np.concatenate([g.colind, np.zeros(1, np.int32)])).to(cuda)
    d_rp = torch.zeros(nb + 1, dtype=torch.int32, device=cuda)
    nt = C.c_int(0)
    assert lib.b2sr_ref_csr2bsr_nnz(d_csr_rp.data_ptr(), d_csr_ci.data_ptr(), g.nrows, g.ncols, T,
                                    d_rp.data_ptr(), C.byref(nt)) == 0
    cap = max(nt.value, nt_cap or 0, 1)
    d_ci = torch.zeros(cap + 64, dtype=torch.int32, device=cuda)
    d_tl = torch.zeros((cap + 64) * T, dtype=torch.from_numpy(np.zeros(1, WORD[T])).dtype, device=cuda)
    rp_h = np.ascontiguousarray(g.rowptr)
    ci_h = np.ascontiguousarray(g.colind)
    assert lib.b2sr_ref_csr2bsr_batch(rp_h.ctypes.data, ci_h.ctypes.data, g.nrows, g.ncols, g.nnz,
                                      d_rp.data_ptr(), d_ci.data_ptr(), d_tl.data_ptr(), T, nb, nt.value) == 0
    return nb, nt.value, d_rp, d_ci, d_tl


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_shims_accumulate_like_the_reference_drivers(pkg, orc, cuda, shim_lib, T):
    lib = shim_lib
    g = pkg.rmat(12, 16, seed=31)
    nb, nt, d_rp, d_ci, d_tl = ref_pack(lib, g, T, cuda)
    n = nb * T
    rng = np.random.default_rng(T)
    x = np.zeros(n, np.float32)
    x[: g.nrows] = rng.random(g.nrows, dtype=np.float32)
    xd = torch.from_numpy(x).to(cuda)
    y = torch.zeros(n, device=cuda)
    xb = (rng.random(g.nrows) < 0.3).astype(np.float32)
    bits = pkg.pack_vec_bits(torch.from_numpy(xb).to(cuda), T)
    ybits = torch.zeros(nb, dtype=bits.dtype, device=cuda)
    ycnt = torch.zeros(n, device=cuda)
    reps = 5  # TEST_TIMES of the reference drivers
    for _ in range(reps):
        assert lib.b2sr_ref_bmv_bin_full_full(T, d_tl.data_ptr(), xd.data_ptr(), y.data_ptr(), d_rp.data_ptr(),
                                              d_ci.data_ptr(), nb) == 0
        assert lib.b2sr_ref_bmv_bin_bin_bin(T, d_tl.data_ptr(), bits.data_ptr(), ybits.data_ptr(), d_rp.data_ptr(),
                                            d_ci.data_ptr(), nb) == 0
        assert lib.b2sr_ref_bmv_bin_bin_full(T, d_tl.data_ptr(), bits.data_ptr(), ycnt.data_ptr(), d_rp.data_ptr(),
                                             d_ci.data_ptr(), nb) == 0
    torch.cuda.synchronize()
    y64 = orc.csr_spmv_f64(g.rowptr, g.colind, g.nrows, x[: g.nrows])
    scale = np.maximum(orc.csr_spmv_abs_f64(g.rowptr, g.colind, g.nrows, x[: g.nrows]), 1e-30)
    err = np.abs(y.cpu().numpy()[: g.nrows].astype(np.float64) - reps * y64) / (reps * scale)
    print(f"T={T}: bin_full_full after {reps} accumulating shim calls, max error vs FP64 {err.max():.2e}")
    assert err.max() <= REL_TOL
    brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
    want_bits = orc.bmv_bin_bin_bin(T, brp, bci, tiles, orc.pack_vec_bits(xb, T))
    assert np.array_equal(to_np_words(ybits, T), want_bits)  # |= is idempotent
    cnt = orc.csr_spmv_count(g.rowptr, g.colind, g.nrows, xb > 0)
    assert np.array_equal(ycnt.cpu().numpy()[: g.nrows], reps * cnt.astype(np.float32))


def test_shim_cache_follows_a_repack_into_the_same_arrays(pkg, orc, cuda, shim_lib):
    lib = shim_lib
    T = 8
    g1 = pkg.rmat(12, 16, seed=41)
    g2 = pkg.erdos_renyi(g1.nrows, 6.0, seed=42)  # same size, other structure, fewer tiles
    nb, nt1, d_rp, d_ci, d_tl = ref_pack(lib, g1, T, cuda)
    x = torch.rand(nb * T, device=cuda)
    xh = x.cpu().numpy()
    for g in (g1, g2):
        if g is g2:  # re-pack g2 into g1's arrays (sized for g1's tile count)
            nt = C.c_int(0)
            d_csr_rp = torch.from_numpy(g.rowptr).to(cuda)
            d_csr_ci = torch.from_numpy(np.concatenate([g.colind, np.zeros(1, np.int32)])).to(cuda)
            assert lib.b2sr_ref_csr2bsr_nnz(d_csr_rp.data_ptr(), d_csr_ci.data_ptr(), g.nrows, g.ncols, T,
                                            d_rp.data_ptr(), C.byref(nt)) == 0
            assert nt.value <= nt1
            rp_h, ci_h = np.ascontiguousarray(g.rowptr), np.ascontiguousarray(g.colind)
            assert lib.b2sr_ref_csr2bsr_batch(rp_h.ctypes.data, ci_h.ctypes.data, g.nrows, g.ncols, g.nnz,
                                              d_rp.data_ptr(), d_ci.data_ptr(), d_tl.data_ptr(), T, nb,
                                              nt.value) == 0
        y = torch.zeros(nb * T, device=cuda)
        assert lib.b2sr_ref_bmv_bin_full_full(T, d_tl.data_ptr(), x.data_ptr(), y.data_ptr(), d_rp.data_ptr(),
                                              d_ci.data_ptr(), nb) == 0
        torch.cuda.synchronize()
        y64 = orc.csr_spmv_f64(g.rowptr, g.colind, g.nrows, xh[: g.nrows])
        scale = np.maximum(orc.csr_spmv_abs_f64(g.rowptr, g.colind, g.nrows, xh[: g.nrows]), 1e-30)
        err = np.abs(y.cpu().numpy()[: g.nrows].astype(np.float64) - y64) / scale
        assert err.max() <= REL_TOL, f"stale plan after re-pack: {err.max():.3e}"
    # an explicit release, then the same arrays again: rebuilt, same result
    lib.b2sr_ref_release(d_rp.data_ptr())
    y2 = torch.zeros(nb * T, device=cuda)
    assert lib.b2sr_ref_bmv_bin_full_full(T, d_tl.data_ptr(), x.data_ptr(), y2.data_ptr(), d_rp.data_ptr(),
                                          d_ci.data_ptr(), nb) == 0
    torch.cuda.synchronize()
    assert torch.equal(y, y2)  # deterministic: bitwise-equal repeats


@pytest.mark.parametrize("T", [4, 8])
def test_shim_costs_what_the_matrix_api_costs_on_rmat20(pkg, cuda, shim_lib, T):
    """R-MAT scale 20: the drivers' timed shim launch within 1.1x of the
    handle API's call (both the row-binned kernels; CUDA events, L2 flushed
    by a 256 MB read before every call)."""
    lib = shim_lib
    g = pkg.rmat(20, 16, 0.57, 0.19, 0.19, 1)
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    desc = pkg._lib.MatrixDesc()
    assert lib.b2sr_matrix_describe(A.handle, C.byref(desc)) == 0
    nb = A.nblockrows
    x = torch.rand(nb * T, device=cuda)
    y_api = torch.zeros(nb * T, device=cuda)
    y_shim = torch.zeros(nb * T, device=cuda)
    flush = torch.empty(64 << 20, device=cuda).uniform_()

    def api():
        A.spmv_bin_full_full(x, y_api, accumulate=True)

    def shim():
        assert lib.b2sr_ref_bmv_bin_full_full(T, desc.d_tiles, x.data_ptr(), y_shim.data_ptr(), desc.d_rowptr,
                                              desc.d_colind, nb) == 0

    def timed(fn, reps=20):
        fn()  # plans built, caches warm
        ts = []
        for _ in range(reps):
            flush.amax()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    t_api, t_shim = timed(api), timed(shim)
    print(f"T={T}: shim {t_shim * 1e3:.1f} us, matrix API {t_api * 1e3:.1f} us per call")
    assert torch.equal(y_api, y_shim)  # same kernels, same accumulation count
    assert t_shim <= 1.1 * t_api
    A.close()
