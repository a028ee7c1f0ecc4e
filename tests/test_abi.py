"""CPU tests of the C ABI boundary: the library loads, exports every function
that include/*.h declares, and rejects bad arguments before touching the GPU."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import pytest


def test_every_declared_symbol_is_exported(pkg):
    lib = pkg._lib.load()
    declared = pkg._lib.declared_functions()
    assert len(declared) >= 30
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, f"declared in include/*.h but not exported: {missing}"
    nm = subprocess.run(["nm", "-D", "--defined-only", pkg.library_path()], capture_output=True,
                        text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in nm.splitlines() if " T " in ln}
    assert set(declared) <= exported


def test_every_exported_symbol_is_declared(pkg):
    nm = subprocess.run(["nm", "-D", "--defined-only", pkg.library_path()], capture_output=True,
                        text=True, check=True).stdout
    ours = {ln.split()[-1] for ln in nm.splitlines() if " T " in ln and ln.split()[-1].startswith("b2sr_")}
    assert ours == set(pkg._lib.declared_functions())


def test_status_strings_and_version(pkg):
    lib = pkg._lib.load()
    assert lib.b2sr_status_string(0) == b"success"
    assert b"CSR" in lib.b2sr_status_string(2)
    assert lib.b2sr_version() >= 10000


@pytest.mark.parametrize("tile", [0, 3, 5, 64, -4])
def test_pack_rejects_bad_tile_size_before_any_cuda_call(pkg, tile):
    lib = pkg._lib.load()
    out = C.c_void_p()
    rc = lib.b2sr_pack_csr(C.c_void_p(16), C.c_void_p(16), 8, 8, 4, tile, None, C.byref(out))
    assert rc == 1 and out.value is None


def test_pack_rejects_null_and_negative_sizes(pkg):
    lib = pkg._lib.load()
    out = C.c_void_p()
    assert lib.b2sr_pack_csr(None, None, 8, 8, 4, 8, None, C.byref(out)) == 1
    assert lib.b2sr_pack_csr(C.c_void_p(16), C.c_void_p(16), -1, 8, 4, 8, None, C.byref(out)) == 1
    assert lib.b2sr_pack_csr(C.c_void_p(16), None, 8, 8, 4, 8, None, C.byref(out)) == 1
    assert lib.b2sr_pack_csr(C.c_void_p(16), C.c_void_p(16), 8, 8, 4, 8, None, None) == 1


def test_vector_and_shim_argument_checks(pkg):
    lib = pkg._lib.load()
    assert lib.b2sr_pack_vec_bits(None, 10, 8, None, None) == 1
    assert lib.b2sr_pack_vec_bits(None, 0, 8, None, None) == 0  # nothing to do
    assert lib.b2sr_unpack_vec_bits(None, 10, 7, None, None) == 1
    assert lib.b2sr_ref_bmv_bin_full_full(6, None, None, None, None, None, 4) == 1
    # with rows to compute, a null tile, x or colind array (or, for FP32, a
    # misaligned x or y) is refused before any CUDA call; never dereferenced
    p = C.c_void_p(4096)
    for fn in (lib.b2sr_ref_bmv_bin_full_full, lib.b2sr_ref_bmv_bin_bin_full, lib.b2sr_ref_bmv_bin_bin_bin):
        assert fn(4, None, p, p, p, p, 8) == 1
        assert fn(4, p, None, p, p, p, 8) == 1
        assert fn(4, p, p, p, p, None, 8) == 1
        assert fn(4, None, None, p, p, None, 0) == 0  # no rows: nothing to do
    assert lib.b2sr_ref_bmv_bin_full_full(4, p, C.c_void_p(4100), p, p, p, 8) == 1
    assert lib.b2sr_ref_bmv_bin_full_full(4, p, p, C.c_void_p(4100), p, p, 8) == 1
    assert lib.b2sr_spmv_bin_full_full_noalloc(4, p, p, p, 8, 32, None, p, 0, None) == 1
    assert lib.b2sr_spmv_bin_full_full_noalloc(4, None, p, p, 8, 32, p, p, 0, None) == 1
    assert lib.b2sr_spmv_bin_full_full_noalloc(4, p, p, None, 8, 32, p, p, 0, None) == 1
    assert lib.b2sr_ref_bmv_bin_bin_bin(8, None, None, None, None, None, 4) == 1
    n = C.c_int()
    assert lib.b2sr_ref_csr2bsr_nnz(None, None, 4, 4, 8, None, C.byref(n)) == 1
    assert lib.b2sr_spmv_bin_full_full(None, None, None, 0, None) == 1
    assert lib.b2sr_matrix_describe(None, None) == 1


def test_header_compiles_as_c_in_the_drop_in_driver(pkg, tmp_path):
    """include/b2sr.h is plain C: the C drop-in driver compiles and links with
    gcc -std=c11 -Wall -Wextra -Werror against it and the built library (run
    on a GPU by tests/test_gpu_c_driver.py)."""
    import shutil
    from pathlib import Path
    cc = shutil.which("gcc") or shutil.which("cc")
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    if cc is None or not (cuda / "include" / "cuda_runtime.h").exists():
        pytest.skip("no C compiler or CUDA headers")
    root = Path(__file__).resolve().parents[1]
    lib_dir = Path(pkg.library_path()).parent
    cmd = [cc, "-std=c11", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{root / 'include'}", f"-I{cuda / 'include'}",
           str(root / "tests" / "c_driver" / "drop_in_driver.c"), "-o", str(tmp_path / "d")]
    cmd += [f"-L{d}" for d in (cuda / "lib64", cuda / "lib") if d.exists()]
    cmd += ["-lcudart", f"-L{lib_dir}", "-lb2sr", "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
