"""numpy face of the C oracle (liboracle.so).  TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py as
the checker; the library never imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_lib = None

WORD = {4: np.uint8, 8: np.uint8, 16: np.uint16, 32: np.uint32}


def _load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    import importlib.util
    spec = importlib.util.spec_from_file_location("_b2sr_oracle_build", HERE / "build_oracle.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    path = mod.build_oracle()
    lib = C.CDLL(str(path))
    P = C.c_void_p
    I = C.c_int
    sig = {
        "oracle_b2sr_structure": (C.c_longlong, [P, P, I, I, P]),
        "oracle_b2sr_fill": (None, [P, P, I, I, P, P, P]),
        "oracle_pack_vec_bits": (None, [P, I, I, P]),
        "oracle_unpack_vec_bits": (None, [P, I, I, P]),
        "oracle_bmv_bin_bin_bin": (None, [I, I, P, P, P, P, P, I]),
        "oracle_bmv_bin_bin_bin_masked": (None, [I, I, P, P, P, P, P, P]),
        "oracle_bmv_bin_bin_full": (None, [I, I, P, P, P, P, P, I]),
        "oracle_bmv_bin_bin_count": (None, [I, I, P, P, P, P, P, I]),
        "oracle_bmv_bin_full_full": (None, [I, I, P, P, P, P, P, I]),
        "oracle_bmv_bin_full_full_f64": (None, [I, I, P, P, P, P, P]),
        "oracle_bmm_f64": (None, [I, I, P, P, P, P, I, I, P, I]),
        "oracle_csr_spmv_f64": (None, [P, P, I, P, P]),
        "oracle_csr_spmv_abs_f64": (None, [P, P, I, P, P]),
        "oracle_csr_spmv_count": (None, [P, P, I, P, P]),
        "oracle_csr_spmv_f32_omp": (I, [P, P, I, P, P, I]),
        "oracle_max_threads": (I, []),
        "oracle_rmat_edges": (None, [I, C.c_longlong, C.c_double, C.c_double, C.c_double, C.c_uint64, P, P]),
        "oracle_sym_csr": (C.c_longlong, [P, P, C.c_longlong, I, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


# ---- packing ------------------------------------------------------------------------
def csr_to_b2sr(rowptr, colind, nrows: int, T: int):
    """(browptr, bcolind, tiles) of the CSR, in the reference layout."""
    rp, ci = _i32(rowptr), _i32(colind)
    if ci.size == 0:
        ci = np.zeros(1, np.int32)
    nb = (nrows + T - 1) // T
    brp = np.zeros(nb + 1, np.int32)
    nt = _load().oracle_b2sr_structure(_p(rp), _p(ci), nrows, T, _p(brp))
    bci = np.zeros(max(nt, 1), np.int32)
    tiles = np.zeros(max(nt * T, 1), WORD[T])
    _load().oracle_b2sr_fill(_p(rp), _p(ci), nrows, T, _p(brp), _p(bci), _p(tiles))
    return brp, bci[:nt], tiles[: nt * T]


def pack_vec_bits(x, T: int) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    n = x.size
    out = np.zeros(max((n + T - 1) // T, 1), WORD[T])
    _load().oracle_pack_vec_bits(_p(x), n, T, _p(out))
    return out[: (n + T - 1) // T]


def unpack_vec_bits(bits, n: int, T: int) -> np.ndarray:
    b = np.ascontiguousarray(bits, dtype=WORD[T])
    out = np.zeros(max(n, 1), np.float32)
    _load().oracle_unpack_vec_bits(_p(b), n, T, _p(out))
    return out[:n]


# ---- multiplies on B2SR -------------------------------------------------------------
def _b2sr_args(T, brp, bci, tiles):
    bci = _i32(bci) if len(bci) else np.zeros(1, np.int32)
    tiles = np.ascontiguousarray(tiles, dtype=WORD[T]) if len(tiles) else np.zeros(T, WORD[T])
    return _i32(brp), bci, tiles


def bmv_bin_bin_bin(T, brp, bci, tiles, xbits, y=None, accumulate=False, nb=None):
    nb = len(brp) - 1 if nb is None else nb
    brp, bci, tiles = _b2sr_args(T, brp, bci, tiles)
    xb = np.ascontiguousarray(xbits, dtype=WORD[T])
    y = np.zeros(max(nb, 1), WORD[T]) if y is None else np.ascontiguousarray(y, dtype=WORD[T]).copy()
    _load().oracle_bmv_bin_bin_bin(T, nb, _p(brp), _p(bci), _p(tiles), _p(xb), _p(y), int(accumulate))
    return y[:nb]


def bmv_bin_bin_bin_masked(T, brp, bci, tiles, xbits, maskbits):
    nb = len(brp) - 1
    brp, bci, tiles = _b2sr_args(T, brp, bci, tiles)
    xb = np.ascontiguousarray(xbits, dtype=WORD[T])
    mb = np.ascontiguousarray(maskbits, dtype=WORD[T])
    y = np.zeros(max(nb, 1), WORD[T])
    _load().oracle_bmv_bin_bin_bin_masked(T, nb, _p(brp), _p(bci), _p(tiles), _p(xb), _p(mb), _p(y))
    return y[:nb]


def bmv_bin_bin_full(T, brp, bci, tiles, xbits, y=None, accumulate=False):
    nb = len(brp) - 1
    brp, bci, tiles = _b2sr_args(T, brp, bci, tiles)
    xb = np.ascontiguousarray(xbits, dtype=WORD[T])
    y = np.zeros(max(nb * T, 1), np.float32) if y is None else np.ascontiguousarray(y, np.float32).copy()
    _load().oracle_bmv_bin_bin_full(T, nb, _p(brp), _p(bci), _p(tiles), _p(xb), _p(y), int(accumulate))
    return y[: nb * T]


def bmv_bin_bin_count(T, brp, bci, tiles, xbits, y=None, accumulate=False):
    nb = len(brp) - 1
    brp, bci, tiles = _b2sr_args(T, brp, bci, tiles)
    xb = np.ascontiguousarray(xbits, dtype=WORD[T])
    y = np.zeros(max(nb * T, 1), np.int32) if y is None else np.ascontiguousarray(y, np.int32).copy()
    _load().oracle_bmv_bin_bin_count(T, nb, _p(brp), _p(bci), _p(tiles), _p(xb), _p(y), int(accumulate))
    return y[: nb * T]


def bmv_bin_full_full(T, brp, bci, tiles, x, y=None, accumulate=False):
    nb = len(brp) - 1
    brp, bci, tiles = _b2sr_args(T, brp, bci, tiles)
    xf = np.ascontiguousarray(x, np.float32)
    y = np.zeros(max(nb * T, 1), np.float32) if y is None else np.ascontiguousarray(y, np.float32).copy()
    _load().oracle_bmv_bin_full_full(T, nb, _p(brp), _p(bci), _p(tiles), _p(xf), _p(y), int(accumulate))
    return y[: nb * T]


def bmv_bin_full_full_f64(T, brp, bci, tiles, x):
    nb = len(brp) - 1
    brp, bci, tiles = _b2sr_args(T, brp, bci, tiles)
    xf = np.ascontiguousarray(x, np.float32)
    y = np.zeros(max(nb * T, 1), np.float64)
    _load().oracle_bmv_bin_full_full_f64(T, nb, _p(brp), _p(bci), _p(tiles), _p(xf), _p(y))
    return y[: nb * T]


def bmm_f64(T, brp, bci, tiles, X):
    nb = len(brp) - 1
    brp, bci, tiles = _b2sr_args(T, brp, bci, tiles)
    X = np.ascontiguousarray(X, np.float64)
    k = X.shape[1]
    Y = np.zeros((max(nb * T, 1), k), np.float64)
    _load().oracle_bmm_f64(T, nb, _p(brp), _p(bci), _p(tiles), _p(X), k, k, _p(Y), k)
    return Y[: nb * T]


# ---- CSR oracle -----------------------------------------------------------------------------
def csr_spmv_f64(rowptr, colind, nrows, x):
    rp, ci = _i32(rowptr), _i32(colind)
    ci = ci if ci.size else np.zeros(1, np.int32)
    xf = np.ascontiguousarray(x, np.float32)
    y = np.zeros(max(nrows, 1), np.float64)
    _load().oracle_csr_spmv_f64(_p(rp), _p(ci), nrows, _p(xf), _p(y))
    return y[:nrows]


def csr_spmv_abs_f64(rowptr, colind, nrows, x):
    rp, ci = _i32(rowptr), _i32(colind)
    ci = ci if ci.size else np.zeros(1, np.int32)
    xf = np.ascontiguousarray(x, np.float32)
    y = np.zeros(max(nrows, 1), np.float64)
    _load().oracle_csr_spmv_abs_f64(_p(rp), _p(ci), nrows, _p(xf), _p(y))
    return y[:nrows]


def csr_spmv_count(rowptr, colind, nrows, xbool):
    rp, ci = _i32(rowptr), _i32(colind)
    ci = ci if ci.size else np.zeros(1, np.int32)
    xb = np.ascontiguousarray(np.asarray(xbool) != 0, dtype=np.uint8)
    y = np.zeros(max(nrows, 1), np.int64)
    _load().oracle_csr_spmv_count(_p(rp), _p(ci), nrows, _p(xb), _p(y))
    return y[:nrows]


def csr_spmv_f32_omp(rowptr, colind, nrows, x, y=None, nthreads=0):
    """The timed CPU baseline.  Returns (y, threads used)."""
    rp, ci = _i32(rowptr), _i32(colind)
    ci = ci if ci.size else np.zeros(1, np.int32)
    xf = np.ascontiguousarray(x, np.float32)
    y = np.zeros(max(nrows, 1), np.float32) if y is None else y
    used = _load().oracle_csr_spmv_f32_omp(_p(rp), _p(ci), nrows, _p(xf), _p(y), nthreads)
    return y[:nrows], used


def max_threads() -> int:
    return _load().oracle_max_threads()


def rmat_csr(scale: int, edge_factor: int, a: float, b: float, c: float, seed: int):
    """The symmetrised, de-duplicated, loop-free R-MAT CSR (rowptr, colind as
    int32) built from oracle_rmat_edges with numpy, without the library: the
    input of the benchmark's CPU arm."""
    n = 1 << scale
    m = edge_factor << scale
    u = np.empty(m, np.int32)
    v = np.empty(m, np.int32)
    _load().oracle_rmat_edges(scale, m, a, b, c, seed, _p(u), _p(v))
    rowptr = np.empty(n + 1, np.int32)
    colind = np.empty(max(2 * m, 1), np.int32)
    nnz = _load().oracle_sym_csr(_p(u), _p(v), m, n, _p(rowptr), _p(colind))
    if nnz < 0:
        raise ValueError("R-MAT graph exceeds the int32 index range")
    return rowptr, colind[:nnz].copy()
