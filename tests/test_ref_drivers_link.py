"""CPU check of the drop-in at link level: the reference's own
bmv_eval/test_bin_full_full.cu, with only its structure pass, packer and timed
launches bound to the C ABI (oracle/ref_drivers.py), compiles for sm_103a and
links against libb2sr.so.  The GPU tests run these drivers."""
from __future__ import annotations

import importlib.util
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_patched_reference_driver_links_against_the_library(pkg, tmp_path):
    spec = importlib.util.spec_from_file_location("b2sr_ref_drivers", ROOT / "oracle" / "ref_drivers.py")
    rd = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(rd)
    if rd.prepare() is None:
        pytest.skip("no reference checkout and no prepared drivers")
    src = (rd.OUT / "test_bin_full_full.cu").read_text()
    assert "b2sr_ref_bmv_bin_full_full(tiledim, tA, fB, fC, bsrRowPtr, bsrColInd, nblockrows);" in src
    assert "bmv4_bin_full_full<<<" not in src and "cusparseXcsr2bsrNnz(" not in src
    exe = tmp_path / "test_bin_full_full_T4"
    res = rd.compile_driver("test_bin_full_full.cu", 4, Path(pkg.library_path()).parent, ROOT / "include", exe)
    assert res.returncode == 0, res.stderr[-3000:]
    undefined = subprocess.run(["nm", "-D", "--undefined-only", str(exe)], capture_output=True, text=True).stdout
    for sym in ("b2sr_ref_bmv_bin_full_full", "b2sr_ref_csr2bsr_nnz", "b2sr_ref_csr2bsr_batch"):
        assert sym in undefined, f"{sym} is not bound to the library"
