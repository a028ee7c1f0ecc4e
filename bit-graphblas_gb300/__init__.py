"""GB300 (sm_103a) B2SR binary SpMV: the Bit-GraphBLAS hot path behind a C ABI.

The compute lives in libb2sr.so (csrc/, C ABI in include/b2sr.h); this package
binds it for Python callers.  The directory name is not a Python identifier,
so load it by path, e.g. ``__graft_entry__.load_package()``, which registers it
as ``bit_graphblas_gb300``.
"""
from . import _lib
from ._lib import B2SRError
from .autograd import B2SRAggregate, SumAggGNN, aggregate
from .graphs import CSR, block_diag, er_batch, erdos_renyi, from_edges, read_mtx, rmat
from .matrix import (TILE_SIZES, VARIANTS, B2SRMatrix, KernelTimer, pack_vec_bits, unpack_vec_bits, word_dtype,
                     word_numpy_dtype)

__all__ = [
    "B2SRAggregate", "B2SRError", "B2SRMatrix", "KernelTimer", "SumAggGNN", "aggregate", "CSR", "TILE_SIZES", "VARIANTS", "block_diag", "er_batch", "erdos_renyi",
    "from_edges", "pack_vec_bits", "read_mtx", "rmat", "unpack_vec_bits", "word_dtype",
    "word_numpy_dtype",
]


def library_path() -> str:
    return str(_lib.LIB_PATH)
