"""ctypes binding of libb2sr.so (the C ABI in include/b2sr.h and include/b2sr_graph.h).

Loading fails loudly when the library has not been built: there is no Python
fallback for any multiply.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libb2sr.so"
INCLUDE = PKG.parent / "include"

c_int_p = C.POINTER(C.c_int)
c_void_p = C.c_void_p


class B2SRError(RuntimeError):
    """A non-success b2sr_status from the C ABI."""

    def __init__(self, status: int, what: str, cuda_error: int = 0):
        self.status = status
        self.cuda_error = cuda_error
        msg = f"{what}: {status_string(status)} (status {status})"
        if cuda_error:
            msg += f", cuda error {cuda_error}"
        super().__init__(msg)


class MatrixDesc(C.Structure):
    _fields_ = [
        ("nrows", C.c_int), ("ncols", C.c_int), ("tile_dim", C.c_int),
        ("nblockrows", C.c_int), ("nblockcols", C.c_int), ("nblocks", C.c_int),
        ("nnz", C.c_longlong),
        ("d_rowptr", c_void_p), ("d_colind", c_void_p), ("d_tiles", c_void_p),
        ("owns_storage", C.c_int),
    ]


class LaunchConfig(C.Structure):
    _fields_ = [("threads", C.c_int), ("items_per_thread", C.c_int), ("ctas_per_sm", C.c_int),
                ("algorithm", C.c_int), ("gather", C.c_int), ("rhs_block", C.c_int), ("direction", C.c_int)]


class TuneResult(C.Structure):
    _fields_ = [("tile_dim", C.c_int), ("algorithm", C.c_int), ("gather", C.c_int), ("threads", C.c_int),
                ("items_per_thread", C.c_int), ("best_ms", C.c_float), ("candidates", C.c_int),
                ("rhs_block", C.c_int)]


class CSRHost(C.Structure):
    _fields_ = [("nrows", C.c_int), ("ncols", C.c_int), ("nnz", C.c_longlong),
                ("rowptr", c_int_p), ("colind", c_int_p)]


ALLOC_FN = C.CFUNCTYPE(c_void_p, C.c_size_t, c_void_p)
FREE_FN = C.CFUNCTYPE(None, c_void_p, c_void_p)

# name -> (restype, argtypes)
_PROTOS = {
    "b2sr_status_string": (C.c_char_p, [C.c_int]),
    "b2sr_last_cuda_error": (C.c_int, []),
    "b2sr_version": (C.c_int, []),
    "b2sr_set_allocator": (None, [ALLOC_FN, FREE_FN, c_void_p]),
    "b2sr_pack_csr": (C.c_int, [c_void_p, c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, c_void_p,
                                C.POINTER(c_void_p)]),
    "b2sr_matrix_wrap": (C.c_int, [c_void_p, c_void_p, c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                   c_void_p, C.POINTER(c_void_p)]),
    "b2sr_matrix_transpose": (C.c_int, [c_void_p, c_void_p, C.POINTER(c_void_p)]),
    "b2sr_matrix_describe": (C.c_int, [c_void_p, C.POINTER(MatrixDesc)]),
    "b2sr_free": (None, [c_void_p]),
    "b2sr_matrix_download": (C.c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "b2sr_pack_vec_bits": (C.c_int, [c_void_p, C.c_int, C.c_int, c_void_p, c_void_p]),
    "b2sr_unpack_vec_bits": (C.c_int, [c_void_p, C.c_int, C.c_int, c_void_p, c_void_p]),
    "b2sr_spmv_bin_bin_bin": (C.c_int, [c_void_p, c_void_p, c_void_p, C.c_int, c_void_p]),
    "b2sr_spmv_bin_bin_full": (C.c_int, [c_void_p, c_void_p, c_void_p, C.c_int, c_void_p]),
    "b2sr_spmv_bin_bin_count": (C.c_int, [c_void_p, c_void_p, c_void_p, C.c_int, c_void_p]),
    "b2sr_spmv_bin_full_full": (C.c_int, [c_void_p, c_void_p, c_void_p, C.c_int, c_void_p]),
    "b2sr_spmv_bin_bin_bin_masked": (C.c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "b2sr_spmv_multi_bits": (C.c_int, [c_void_p, c_void_p, c_void_p, C.c_int, c_void_p, C.c_int, c_void_p]),
    "b2sr_spmm_bin_full_full": (C.c_int, [c_void_p, c_void_p, C.c_int, C.c_longlong, c_void_p, C.c_longlong,
                                          C.c_int, c_void_p]),
    "b2sr_spmm_bin_full_full_f64": (C.c_int, [c_void_p, c_void_p, C.c_int, C.c_longlong, c_void_p,
                                              C.c_longlong, C.c_int, c_void_p]),
    "b2sr_matrix_set_launch": (C.c_int, [c_void_p, C.c_int, C.POINTER(LaunchConfig)]),
    "b2sr_matrix_get_launch": (C.c_int, [c_void_p, C.c_int, C.POINTER(LaunchConfig)]),
    "b2sr_last_launch_count": (C.c_int, []),
    "b2sr_matrix_save": (C.c_int, [c_void_p, C.c_char_p]),
    "b2sr_matrix_load": (C.c_int, [C.c_char_p, c_void_p, C.POINTER(c_void_p)]),
    "b2sr_kernel_timer_start": (C.c_int, [C.c_int]),
    "b2sr_kernel_timer_read": (C.c_int, [C.POINTER(C.c_float), C.c_int]),
    "b2sr_autotune": (C.c_int, [c_void_p, c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, c_void_p, C.c_int,
                                c_void_p, C.POINTER(c_void_p), C.POINTER(TuneResult)]),
    "b2sr_autotune_clear_cache": (None, []),
    "b2sr_spmv_bin_full_full_noalloc": (C.c_int, [C.c_int, c_void_p, c_void_p, c_void_p, C.c_int, C.c_int,
                                                  c_void_p, c_void_p, C.c_int, c_void_p]),
    "b2sr_ref_csr2bsr_nnz": (C.c_int, [c_void_p, c_void_p, C.c_int, C.c_int, C.c_int, c_void_p, c_int_p]),
    "b2sr_ref_csr2bsr_batch": (C.c_int, [c_void_p, c_void_p, C.c_int, C.c_int, C.c_int, c_void_p,
                                         c_void_p, c_void_p, C.c_int, C.c_int, C.c_int]),
    "b2sr_ref_bmv_bin_bin_bin": (C.c_int, [C.c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, C.c_int]),
    "b2sr_ref_bmv_bin_bin_full": (C.c_int, [C.c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, C.c_int]),
    "b2sr_ref_bmv_bin_full_full": (C.c_int, [C.c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, C.c_int]),
    "b2sr_ref_release": (None, [c_void_p]),
    # graph ingest
    "b2sr_graph_coo_to_csr": (C.c_int, [c_void_p, c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_int,
                                        C.c_int, C.POINTER(CSRHost)]),
    "b2sr_graph_rmat": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                  C.POINTER(CSRHost)]),
    "b2sr_graph_er": (C.c_int, [C.c_int, C.c_longlong, C.c_uint64, C.POINTER(CSRHost)]),
    "b2sr_graph_er_batch": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_uint64,
                                      C.POINTER(CSRHost), c_void_p, c_void_p, c_void_p]),
    "b2sr_graph_block_diag": (C.c_int, [C.POINTER(CSRHost), c_void_p, C.c_int, C.POINTER(CSRHost)]),
    "b2sr_graph_read_mtx": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(CSRHost)]),
    "b2sr_graph_uniform": (None, [C.c_uint64, C.c_longlong, C.c_longlong, c_void_p]),
    "b2sr_graph_free": (None, [C.POINTER(CSRHost)]),
}

_lib = None


def declared_functions() -> list[str]:
    """Every function name declared in include/*.h."""
    names = []
    for h in sorted(INCLUDE.glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(b2sr_[a-z0-9_]+)\s*\(", text):
            names.append(m.group(1))
    # typedef'd function pointer names are not functions
    return sorted(set(n for n in names if not n.endswith("_fn")))


def load(path: Path | None = None) -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"libb2sr.so is not built ({p}); run __graft_entry__.build() first")
    lib = C.CDLL(str(p))
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(status: int) -> str:
    try:
        return load().b2sr_status_string(status).decode()
    except Exception:  # library not loadable: still format the number
        return "status"


def check(status: int, what: str) -> None:
    if status != 0:
        raise B2SRError(status, what, load().b2sr_last_cuda_error())
