"""Host graph ingest: canonical CSR (numpy int32) from generators, edge lists or .mtx files.

Thin wrappers over include/b2sr_graph.h.  The canonical form is the one the
reference's readMtx builds (bmv_eval/backend/readMtx.hpp:152-218, 248-306):
mirrored when symmetric, self-loops and duplicates removed, rows sorted.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass
class CSR:
    nrows: int
    ncols: int
    rowptr: np.ndarray  # int32, nrows + 1
    colind: np.ndarray  # int32, nnz

    @property
    def nnz(self) -> int:
        return int(self.colind.size)

    def degrees(self) -> np.ndarray:
        return np.diff(self.rowptr)


def _take(h: _lib.CSRHost) -> CSR:
    lib = _lib.load()
    try:
        n, nnz = h.nrows, h.nnz
        rp = np.ctypeslib.as_array(h.rowptr, shape=(n + 1,)).copy() if n >= 0 else np.zeros(1, np.int32)
        ci = (np.ctypeslib.as_array(h.colind, shape=(nnz,)).copy() if nnz > 0
              else np.zeros(0, np.int32))
        return CSR(n, h.ncols, rp.astype(np.int32, copy=False), ci.astype(np.int32, copy=False))
    finally:
        lib.b2sr_graph_free(C.byref(h))


def _checked(rc: int, what: str) -> None:
    if rc != 0:
        raise ValueError(f"{what} failed with code {rc}")


def rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         seed: int = 1) -> CSR:
    """Symmetrised R-MAT graph without self-loops or duplicates (no noise, no relabelling)."""
    h = _lib.CSRHost()
    _checked(_lib.load().b2sr_graph_rmat(scale, edge_factor, a, b, c, seed, C.byref(h)), "rmat")
    return _take(h)


def erdos_renyi(n: int, avg_degree: float, seed: int = 1) -> CSR:
    """Exactly m = round(n * avg_degree / 2) distinct undirected edges, mirrored (nnz = 2m)."""
    m = int(round(n * avg_degree / 2))
    h = _lib.CSRHost()
    _checked(_lib.load().b2sr_graph_er(n, m, seed, C.byref(h)), "erdos_renyi")
    return _take(h)


def from_edges(rows, cols, nrows: int, ncols: int | None = None, symmetrize: bool = False,
               drop_self_loops: bool = True) -> CSR:
    ncols = nrows if ncols is None else ncols
    r = np.ascontiguousarray(rows, dtype=np.int32)
    c = np.ascontiguousarray(cols, dtype=np.int32)
    h = _lib.CSRHost()
    rc = _lib.load().b2sr_graph_coo_to_csr(
        r.ctypes.data_as(C.c_void_p), c.ctypes.data_as(C.c_void_p), r.size, nrows, ncols,
        int(symmetrize), int(drop_self_loops), C.byref(h))
    _checked(rc, "from_edges")
    return _take(h)


def block_diag(graphs: list[CSR], align: int = 1) -> tuple[CSR, np.ndarray]:
    """Stack graphs block-diagonally; graph g's vertices start at offsets[g], a multiple of `align`."""
    offs = [0]
    for g in graphs:
        offs.append(offs[-1] + (g.nrows + align - 1) // align * align)
    offsets = np.asarray(offs, dtype=np.int32)
    hs = (_lib.CSRHost * max(len(graphs), 1))()
    for i, g in enumerate(graphs):
        hs[i].nrows, hs[i].ncols, hs[i].nnz = g.nrows, g.ncols, g.nnz
        hs[i].rowptr = g.rowptr.ctypes.data_as(_lib.c_int_p)
        hs[i].colind = g.colind.ctypes.data_as(_lib.c_int_p)
    h = _lib.CSRHost()
    rc = _lib.load().b2sr_graph_block_diag(hs, offsets.ctypes.data_as(C.c_void_p), len(graphs), C.byref(h))
    _checked(rc, "block_diag")
    return _take(h), offsets


def er_batch(count: int, n_min: float = 64, n_max: float = 65536, deg_min: float = 4, deg_max: float = 32,
             align: int = 32, seed: int = 4) -> tuple[CSR, np.ndarray, np.ndarray, np.ndarray]:
    """Uneven batch of Erdos-Renyi graphs stacked block-diagonally.

    Returns (stacked CSR, offsets[count+1], sizes[count], degrees[count])."""
    offsets = np.zeros(count + 1, np.int32)
    sizes = np.zeros(count, np.int32)
    degrees = np.zeros(count, np.float64)
    h = _lib.CSRHost()
    rc = _lib.load().b2sr_graph_er_batch(count, n_min, n_max, deg_min, deg_max, align, seed, C.byref(h),
                                        offsets.ctypes.data_as(C.c_void_p), sizes.ctypes.data_as(C.c_void_p),
                                        degrees.ctypes.data_as(C.c_void_p))
    _checked(rc, "er_batch")
    return _take(h), offsets, sizes, degrees


def read_mtx(path: str, drop_self_loops: bool = True) -> CSR:
    h = _lib.CSRHost()
    rc = _lib.load().b2sr_graph_read_mtx(str(path).encode(), int(drop_self_loops), C.byref(h))
    _checked(rc, f"read_mtx({path})")
    return _take(h)


def uniform_stream(seed: int, first: int, count: int) -> np.ndarray:
    out = np.empty(count, np.float64)
    _lib.load().b2sr_graph_uniform(seed, first, count, out.ctypes.data_as(C.c_void_p))
    return out
