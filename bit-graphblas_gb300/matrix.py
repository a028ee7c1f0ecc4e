"""B2SRMatrix: the Python face of the C ABI (include/b2sr.h).

Device memory, streams and tensors come from PyTorch; all compute runs in
libb2sr.so.  Every multiply launches the library's CUDA kernels on the current
torch stream; a missing library raises instead of falling back.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

TILE_SIZES = (4, 8, 16, 32)
VARIANTS = {"bin_bin_bin": 0, "bin_bin_full": 1, "bin_full_full": 2, "bin_bin_count": 3}


def word_dtype(tile_dim: int) -> torch.dtype:
    """Torch dtype holding one tile row / bit-vector word (bit pattern)."""
    return {4: torch.uint8, 8: torch.uint8, 16: torch.int16, 32: torch.int32}[tile_dim]


def word_numpy_dtype(tile_dim: int):
    return {4: np.uint8, 8: np.uint8, 16: np.uint16, 32: np.uint32}[tile_dim]


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def _stream(stream=None) -> int:
    s = torch.cuda.current_stream() if stream is None else stream
    return s.cuda_stream


def _cuda_i32(a, device) -> torch.Tensor:
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=torch.int32).contiguous()
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).to(device)


class B2SRMatrix:
    """A binary matrix in B2SR form on one GPU."""

    def __init__(self, handle: int, owner=None, keep=()):
        self._h = C.c_void_p(handle)
        self._owner = owner  # a transpose keeps its parent alive
        self._keep = keep    # wrapped tensors that must outlive the handle
        d = _lib.MatrixDesc()
        _lib.check(_lib.load().b2sr_matrix_describe(self._h, C.byref(d)), "b2sr_matrix_describe")
        self.nrows, self.ncols, self.tile_dim = d.nrows, d.ncols, d.tile_dim
        self.nblockrows, self.nblockcols, self.nblocks = d.nblockrows, d.nblockcols, d.nblocks
        self.nnz = d.nnz
        self.device = torch.device("cuda", torch.cuda.current_device())

    # ---- construction -------------------------------------------------------------
    @classmethod
    def from_csr(cls, rowptr, colind, nrows: int, ncols: int, tile_dim: int, device=None,
                 stream=None) -> "B2SRMatrix":
        """Pack a CSR (numpy or torch, int32, sorted rows) into B2SR on the device."""
        if tile_dim not in TILE_SIZES:
            raise ValueError(f"tile_dim must be one of {TILE_SIZES}")
        device = torch.device("cuda") if device is None else torch.device(device)
        rp = _cuda_i32(rowptr, device)
        ci = _cuda_i32(colind, device)
        if ci.numel() == 0:
            ci = torch.zeros(1, dtype=torch.int32, device=device)
            nnz = 0
        else:
            nnz = int(ci.numel())
        out = C.c_void_p()
        with torch.cuda.device(device):
            rc = _lib.load().b2sr_pack_csr(rp.data_ptr(), ci.data_ptr(), nrows, ncols, nnz, tile_dim,
                                           _stream(stream), C.byref(out))
            _lib.check(rc, "b2sr_pack_csr")
            return cls(out.value)

    @classmethod
    def autotuned(cls, g, variant: str = "bin_full_full", k: int = 0, tile_dims=(4, 8, 16, 32),
                  device=None) -> tuple["B2SRMatrix", dict]:
        """Pack `g` at the tile size / launch option the autotuner finds fastest
        for `variant` (k > 0: the dense-RHS product with k columns)."""
        device = torch.device("cuda") if device is None else torch.device(device)
        rp = _cuda_i32(g.rowptr, device)
        ci = _cuda_i32(g.colind if g.nnz else np.zeros(1, np.int32), device)
        tds = (C.c_int * len(tile_dims))(*tile_dims)
        out = C.c_void_p()
        res = _lib.TuneResult()
        with torch.cuda.device(device):
            rc = _lib.load().b2sr_autotune(rp.data_ptr(), ci.data_ptr(), g.nrows, g.ncols, g.nnz, VARIANTS[variant], k,
                                           tds, len(tile_dims), _stream(), C.byref(out), C.byref(res))
            _lib.check(rc, "b2sr_autotune")
            info = {f: getattr(res, f) for f, _ in _lib.TuneResult._fields_}
            return cls(out.value), info

    @classmethod
    def from_graph(cls, g, tile_dim: int, device=None) -> "B2SRMatrix":
        return cls.from_csr(g.rowptr, g.colind, g.nrows, g.ncols, tile_dim, device)

    @classmethod
    def wrap(cls, rowptr: torch.Tensor, colind: torch.Tensor, tiles: torch.Tensor, nrows: int,
             ncols: int, tile_dim: int) -> "B2SRMatrix":
        """Borrow existing device B2SR arrays (e.g. built by the reference packer)."""
        nblocks = int(colind.numel())
        out = C.c_void_p()
        rc = _lib.load().b2sr_matrix_wrap(rowptr.data_ptr(), colind.data_ptr() if nblocks else None,
                                          tiles.data_ptr() if nblocks else None, nrows, ncols,
                                          nblocks, tile_dim, _stream(), C.byref(out))
        _lib.check(rc, "b2sr_matrix_wrap")
        return cls(out.value, keep=(rowptr, colind, tiles))

    def save(self, path) -> None:
        """Write the packed matrix to `path` (b2sr_matrix_save: header, checksum, arrays)."""
        _lib.check(_lib.load().b2sr_matrix_save(self._h, str(path).encode()), "b2sr_matrix_save")

    @classmethod
    def load(cls, path, device=None) -> "B2SRMatrix":
        """Read a matrix written by save(); the file's checksum and structure are checked."""
        device = torch.device("cuda") if device is None else torch.device(device)
        out = C.c_void_p()
        with torch.cuda.device(device):
            _lib.check(_lib.load().b2sr_matrix_load(str(path).encode(), _stream(), C.byref(out)), "b2sr_matrix_load")
            return cls(out.value)

    def close(self) -> None:
        if self._h and self._h.value and self._owner is None:
            _lib.load().b2sr_free(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # ---- structure ------------------------------------------------------------------
    def download(self):
        """(rowptr, colind, tiles) as numpy arrays (tiles as uint8/uint16/uint32 words)."""
        rp = np.empty(self.nblockrows + 1, np.int32)
        ci = np.empty(max(self.nblocks, 1), np.int32)
        tl = np.empty(max(self.nblocks * self.tile_dim, 1), word_numpy_dtype(self.tile_dim))
        rc = _lib.load().b2sr_matrix_download(self._h, rp.ctypes.data, ci.ctypes.data, tl.ctypes.data)
        _lib.check(rc, "b2sr_matrix_download")
        return rp, ci[: self.nblocks], tl[: self.nblocks * self.tile_dim]

    def transpose(self) -> "B2SRMatrix":
        out = C.c_void_p()
        rc = _lib.load().b2sr_matrix_transpose(self._h, _stream(), C.byref(out))
        _lib.check(rc, "b2sr_matrix_transpose")
        return B2SRMatrix(out.value, owner=self)

    ALGORITHMS = {"auto": 0, "merge": 1, "rowbin": 2}
    GATHERS = {"auto": 0, "ldg": 1, "texture": 2, "sparse": 3}
    DIRECTIONS = {"pull": 0, "auto": 1, "push": 2}

    def set_launch(self, variant: str, threads: int = 0, items_per_thread: int = 0,
                   ctas_per_sm: int = 0, algorithm: str = "auto", gather: str = "auto",
                   rhs_block: int = 0, direction: str = "pull") -> None:
        """Launch options of later multiplies of `variant`.  direction (bit-vector
        variants): "pull" visits every tile-row; "push" visits only the tile-columns
        with a non-zero x word, through the cached transpose; "auto" chooses per
        call on the device (push when those hold under 18/27/45/85% of the tiles
        at T = 4/8/16/32)."""
        cfg = _lib.LaunchConfig(threads, items_per_thread, ctas_per_sm, self.ALGORITHMS[algorithm],
                                self.GATHERS[gather], rhs_block, self.DIRECTIONS[direction])
        _lib.check(_lib.load().b2sr_matrix_set_launch(self._h, VARIANTS[variant], C.byref(cfg)),
                   "b2sr_matrix_set_launch")

    def get_launch(self, variant: str) -> tuple[int, int, int, str, str, int, str]:
        """(threads, items_per_thread, ctas_per_sm, algorithm, gather, rhs_block, direction)."""
        cfg = _lib.LaunchConfig()
        _lib.check(_lib.load().b2sr_matrix_get_launch(self._h, VARIANTS[variant], C.byref(cfg)),
                   "b2sr_matrix_get_launch")
        algo = {v: k for k, v in self.ALGORITHMS.items()}[cfg.algorithm]
        gather = {v: k for k, v in self.GATHERS.items()}[cfg.gather]
        direction = {v: k for k, v in self.DIRECTIONS.items()}[cfg.direction]
        return cfg.threads, cfg.items_per_thread, cfg.ctas_per_sm, algo, gather, cfg.rhs_block, direction

    # ---- vectors ----------------------------------------------------------------------
    def padded_rows(self) -> int:
        return self.nblockrows * self.tile_dim

    def pack_bits(self, x: torch.Tensor, n: int | None = None) -> torch.Tensor:
        return pack_vec_bits(x, self.tile_dim, n)

    def unpack_bits(self, bits: torch.Tensor, n: int) -> torch.Tensor:
        return unpack_vec_bits(bits, self.tile_dim, n)

    # ---- multiplies ------------------------------------------------------------------------
    def _out(self, y, shape, dtype):
        if y is None:
            return torch.empty(shape, dtype=dtype, device=self.device)
        if y.dtype != dtype or y.numel() < shape or not y.is_contiguous():
            raise ValueError(f"output must be a contiguous {dtype} tensor with >= {shape} elements")
        return y

    def spmv_bin_full_full(self, x: torch.Tensor, y: torch.Tensor | None = None,
                           accumulate: bool = False) -> torch.Tensor:
        """y = A.x in FP32 (y has nblockrows*T entries; rows past nrows are zero)."""
        if x.dtype != torch.float32 or x.numel() < self.ncols or not x.is_contiguous():
            raise ValueError("x must be a contiguous float32 tensor with >= ncols entries")
        y = self._out(y, self.padded_rows(), torch.float32)
        rc = _lib.load().b2sr_spmv_bin_full_full(self._h, x.data_ptr(), y.data_ptr(), int(accumulate),
                                                 _stream())
        _lib.check(rc, "b2sr_spmv_bin_full_full")
        return y

    def _check_bits(self, xbits: torch.Tensor, nwords: int) -> None:
        if xbits.dtype != word_dtype(self.tile_dim) or xbits.numel() < nwords or not xbits.is_contiguous():
            raise ValueError(f"bit vector must be contiguous {word_dtype(self.tile_dim)} with >= {nwords} words")

    def spmm(self, X: torch.Tensor, Y: torch.Tensor | None = None, accumulate: bool = False) -> torch.Tensor:
        """Y = A . X for a dense X [ncols, k] (float32 or float64, row-major, unit
        column stride); Y has nblockrows*T rows (rows past nrows are zero)."""
        if X.dim() != 2 or X.shape[0] < self.ncols or X.stride(1) != 1:
            raise ValueError("X must be [>= ncols, k] with unit column stride")
        if X.dtype not in (torch.float32, torch.float64):
            raise ValueError("X must be float32 or float64")
        k = X.shape[1]
        if Y is None:
            Y = torch.empty((self.padded_rows(), k), dtype=X.dtype, device=self.device)
        if Y.dtype != X.dtype or Y.dim() != 2 or Y.shape[0] < self.padded_rows() or Y.shape[1] != k or Y.stride(1) != 1:
            raise ValueError("Y must be [>= nblockrows*T, k] of X's dtype with unit column stride")
        fn = (_lib.load().b2sr_spmm_bin_full_full if X.dtype == torch.float32
              else _lib.load().b2sr_spmm_bin_full_full_f64)
        rc = fn(self._h, X.data_ptr(), k, X.stride(0), Y.data_ptr(), Y.stride(0), int(accumulate), _stream())
        _lib.check(rc, "b2sr_spmm_bin_full_full")
        return Y

    def spmv_multi_bits(self, X: torch.Tensor, Y: torch.Tensor | None = None, mask: torch.Tensor | None = None,
                        accumulate: bool = False) -> torch.Tensor:
        """32 or 64 frontiers at once: X holds one int32/int64 word per vertex (bit f =
        frontier f); Y[v] = OR of X[u] over the neighbours u of v, AND NOT mask[v]."""
        if X.dtype not in (torch.int32, torch.int64) or X.numel() < self.ncols or not X.is_contiguous():
            raise ValueError("X must be a contiguous int32/int64 tensor with >= ncols words")
        Y = self._out(Y, self.padded_rows(), X.dtype)
        if mask is not None and (mask.dtype != X.dtype or mask.numel() < self.padded_rows()):
            raise ValueError("mask must match X's dtype with >= nblockrows*T words")
        rc = _lib.load().b2sr_spmv_multi_bits(self._h, X.data_ptr(), Y.data_ptr(), 8 * X.element_size(),
                                              None if mask is None else mask.data_ptr(), int(accumulate),
                                              _stream())
        _lib.check(rc, "b2sr_spmv_multi_bits")
        return Y

    def spmv_bin_bin_full(self, xbits: torch.Tensor, y: torch.Tensor | None = None,
                          accumulate: bool = False) -> torch.Tensor:
        self._check_bits(xbits, self.nblockcols)
        y = self._out(y, self.padded_rows(), torch.float32)
        rc = _lib.load().b2sr_spmv_bin_bin_full(self._h, xbits.data_ptr(), y.data_ptr(), int(accumulate),
                                                _stream())
        _lib.check(rc, "b2sr_spmv_bin_bin_full")
        return y

    def spmv_bin_bin_count(self, xbits: torch.Tensor, y: torch.Tensor | None = None,
                           accumulate: bool = False) -> torch.Tensor:
        self._check_bits(xbits, self.nblockcols)
        y = self._out(y, self.padded_rows(), torch.int32)
        rc = _lib.load().b2sr_spmv_bin_bin_count(self._h, xbits.data_ptr(), y.data_ptr(), int(accumulate),
                                                 _stream())
        _lib.check(rc, "b2sr_spmv_bin_bin_count")
        return y

    def spmv_bin_bin_bin(self, xbits: torch.Tensor, y: torch.Tensor | None = None,
                         accumulate: bool = False) -> torch.Tensor:
        self._check_bits(xbits, self.nblockcols)
        y = self._out(y, self.nblockrows, word_dtype(self.tile_dim))
        rc = _lib.load().b2sr_spmv_bin_bin_bin(self._h, xbits.data_ptr(), y.data_ptr(), int(accumulate),
                                               _stream())
        _lib.check(rc, "b2sr_spmv_bin_bin_bin")
        return y

    def spmv_bin_bin_bin_masked(self, xbits: torch.Tensor, maskbits: torch.Tensor,
                                y: torch.Tensor | None = None) -> torch.Tensor:
        self._check_bits(xbits, self.nblockcols)
        self._check_bits(maskbits, self.nblockrows)
        y = self._out(y, self.nblockrows, word_dtype(self.tile_dim))
        rc = _lib.load().b2sr_spmv_bin_bin_bin_masked(self._h, xbits.data_ptr(), maskbits.data_ptr(),
                                                      y.data_ptr(), _stream())
        _lib.check(rc, "b2sr_spmv_bin_bin_bin_masked")
        return y


class KernelTimer:
    """CUDA-event durations of the dominant kernel of each multiply call made
    while the timer is armed (events recorded by the library on the launching
    stream, so the carry fix-up and host enqueue time are excluded)."""

    def __init__(self, capacity: int):
        self.capacity = int(capacity)
        self.ms: list[float] = []

    def __enter__(self) -> "KernelTimer":
        _lib.check(_lib.load().b2sr_kernel_timer_start(self.capacity), "b2sr_kernel_timer_start")
        return self

    def __exit__(self, *exc) -> None:
        buf = (C.c_float * max(self.capacity, 1))()
        n = _lib.load().b2sr_kernel_timer_read(buf, self.capacity)
        if n < 0:
            raise _lib.B2SRError(3, "b2sr_kernel_timer_read", _lib.load().b2sr_last_cuda_error())
        self.ms = [float(buf[i]) for i in range(n)]


def pack_vec_bits(x: torch.Tensor, tile_dim: int, n: int | None = None) -> torch.Tensor:
    """x > 0 as B2SR bit words (ceil(n/T) words, MSB first)."""
    if x.dtype != torch.float32 or not x.is_contiguous():
        raise ValueError("x must be a contiguous float32 tensor")
    n = x.numel() if n is None else n
    out = torch.empty(max((n + tile_dim - 1) // tile_dim, 1), dtype=word_dtype(tile_dim), device=x.device)
    rc = _lib.load().b2sr_pack_vec_bits(x.data_ptr(), n, tile_dim, out.data_ptr(), _stream())
    _lib.check(rc, "b2sr_pack_vec_bits")
    return out


def unpack_vec_bits(bits: torch.Tensor, tile_dim: int, n: int) -> torch.Tensor:
    out = torch.empty(max(n, 1), dtype=torch.float32, device=bits.device)
    rc = _lib.load().b2sr_unpack_vec_bits(bits.data_ptr(), n, tile_dim, out.data_ptr(), _stream())
    _lib.check(rc, "b2sr_unpack_vec_bits")
    return out[:n]
