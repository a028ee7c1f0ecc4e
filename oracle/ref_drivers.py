"""The reference's own timing drivers relinked against libb2sr (test
infrastructure: the drop-in check of the C ABI).

prepare(): copies bmv_eval/test_bin_full_full.cu and test_bin_bin_bin.cu from
    the reference checkout into oracle/_ref/drivers/ with exactly the edits a
    maintainer makes to link them against libb2sr -- the structure pass, the
    packer, the vector packer and the timed kernel launches call the C ABI
    (include/b2sr.h) -- plus one added dump of x and y for the tests.  The
    backend headers the drivers include are copied beside them unchanged.
    Needs the reference checkout (B2SR_REFERENCE_ROOT); elsewhere the prepared
    files are used as they are.
compile_driver(): builds one prepared driver for sm_103a in timing mode
    (-DTILEDIM=T, no VERIFY/BASELINE) and links it against libb2sr.so.

Every edit is a literal pattern that must match the reference file the
stated number of times (a changed reference fails loudly instead of
half-patching).
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref" / "drivers"
REFERENCE_EVAL = Path(os.environ.get("B2SR_REFERENCE_ROOT", "/root/reference")) / "bmv_eval"
DRIVERS = ("test_bin_full_full.cu", "test_bin_bin_bin.cu")
BACKEND = ("bsrbmv.cu", "csr2bsr_batch_bsrbmv.cu", "utility.cu", "readMtx.hpp", "mmio.hpp")

_INCLUDE = ('#include "backend/csr2bsr_batch_bsrbmv.cu"\n',
            '#include "backend/csr2bsr_batch_bsrbmv.cu"\n#include "b2sr.h"\n')
# cusparseXcsr2bsrNnz (test_bin_full_full.cu:189-190, test_bin_bin_bin.cu:208-209)
_NNZ = (re.compile(r"cusparseXcsr2bsrNnz\(handle, dirA, nrows, ncols, csr_descr,\s*"
                   r"csrRowPtr, csrColInd, tiledim, bsr_descr, bsrRowPtr, &nblocks\);"),
        "b2sr_ref_csr2bsr_nnz(csrRowPtr, csrColInd, nrows, ncols, tiledim, bsrRowPtr, &nblocks);")
# csr2bsr_batch_{T} (test_bin_full_full.cu:196-208)
_PACK = (re.compile(r"csr2bsr_batch_(4|8|16|32)\(h_csrRowPtr, h_csrColInd, nrows, ncols, nnz,\s*"
                    r"bsrRowPtr, bsrColInd, tA, tiledim, nblockrows, nblocks\);"),
         "b2sr_ref_csr2bsr_batch(h_csrRowPtr, h_csrColInd, nrows, ncols, nnz, bsrRowPtr, bsrColInd, tA, "
         "tiledim, nblockrows, nblocks);")
# the timed launches of evalHSBSFBmv (test_bin_full_full.cu:285-297, test_bin_bin_bin.cu:358-369)
_LAUNCH = {
    "test_bin_full_full.cu": (re.compile(r"bmv(4|8|16|32)_bin_full_full<<<grid, 1024>>>\(tA, fB, fC, "
                                         r"bsrRowPtr, bsrColInd, nblockrows\);"),
                              "b2sr_ref_bmv_bin_full_full(tiledim, tA, fB, fC, bsrRowPtr, bsrColInd, nblockrows);"),
    "test_bin_bin_bin.cu": (re.compile(r"bmv(4|8|16|32)_bin_bin_bin<<<grid, (32|1024)>>>\(tA, tB, fC, "
                                       r"bsrRowPtr, bsrColInd, nblockrows\);"),
                            "b2sr_ref_bmv_bin_bin_bin(tiledim, tA, tB, fC, bsrRowPtr, bsrColInd, nblockrows);"),
}
# ToBit{T}Row in packRandVec (test_bin_bin_bin.cu:256-281)
_TOBIT = (re.compile(r"ToBit(4|8|16|32)Row<float><<<grid, 32>>>\(fB, tB, nblockrows\);"),
          "b2sr_pack_vec_bits(fB, nblockrows * tiledim, tiledim, tB, 0);")
# The added dump: x (host B) and y after the timed launches, to the file named
# by B2SR_DUMP; y words are written as they are (float, or the tile word type).
_DUMP_FN = """
#include <stdio.h>
#include <stdlib.h>
static void b2sr_dump_result(const void* d_y, size_t y_bytes)
{
    const char* path = getenv("B2SR_DUMP");
    if (!path) return;
    FILE* f = fopen(path, "wb");
    if (!f) return;
    void* h = malloc(y_bytes);
    cudaMemcpy(h, d_y, y_bytes, cudaMemcpyDeviceToHost);
    int hdr[3] = {nrows, nblockrows, tiledim};
    fwrite(hdr, sizeof(int), 3, f);
    fwrite(B, sizeof(float), nrows, f);
    fwrite(h, 1, y_bytes, f);
    fclose(f);
    free(h);
}

void CSR2HSBSF()"""
_Y_BYTES = {"test_bin_full_full.cu": "(size_t)nblockrows * tiledim * sizeof(float)",
            "test_bin_bin_bin.cu": "(size_t)nblockrows * (tiledim <= 8 ? 1 : tiledim / 8)"}


def reference_present() -> bool:
    return all((REFERENCE_EVAL / d).exists() for d in DRIVERS)


def _sub_each(text: str, pat: re.Pattern, repl: str, what: str, count: int) -> str:
    new, n = pat.subn(repl, text)
    if n != count:
        raise RuntimeError(f"{what}: expected {count} matches in the reference driver, found {n}")
    return new


def patch(name: str, text: str) -> str:
    """The driver's text with the drop-in edits applied."""
    if text.count(_INCLUDE[0]) != 1 or text.count("void CSR2HSBSF()") != 1:
        raise RuntimeError(f"{name}: include line or CSR2HSBSF not found exactly once")
    text = text.replace(_INCLUDE[0], _INCLUDE[1])
    text = text.replace("void CSR2HSBSF()", _DUMP_FN, 1)
    text = _sub_each(text, *_NNZ, "cusparseXcsr2bsrNnz", 1)
    text = _sub_each(text, *_PACK, "csr2bsr_batch_{T}", 4)
    text = _sub_each(text, *_LAUNCH[name], "kernel launch", 4)
    if name == "test_bin_bin_bin.cu":
        text = _sub_each(text, *_TOBIT, "ToBit{T}Row", 4)
    call = "    double time = evalHSBSFBmv();\n"
    if text.count(call) != 1:
        raise RuntimeError(f"{name}: timing-mode evalHSBSFBmv call not found exactly once")
    text = text.replace(call, call + f"    b2sr_dump_result(fC, {_Y_BYTES[name]});\n")
    return text


def prepare() -> Path | None:
    """Writes the patched drivers (and the unchanged backend files they
    include) into oracle/_ref/drivers/; returns that folder, or None when
    neither the checkout nor prepared files exist."""
    if not reference_present():
        return OUT if all((OUT / d).exists() for d in DRIVERS) else None
    (OUT / "backend").mkdir(parents=True, exist_ok=True)
    for b in BACKEND:
        shutil.copyfile(REFERENCE_EVAL / "backend" / b, OUT / "backend" / b)
    for d in DRIVERS:
        (OUT / d).write_text(patch(d, (REFERENCE_EVAL / d).read_text()))
    return OUT


def compile_driver(name: str, T: int, lib_dir: Path, include_dir: Path, out: Path) -> subprocess.CompletedProcess:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-w", f"-DTILEDIM={T}",
           "-I", str(include_dir), "-I", str(OUT), str(OUT / name), "-o", str(out),
           "-L", str(lib_dir), "-lb2sr", "-Xlinker", f"-rpath={lib_dir}", "-lcusparse", "-lcublas"]
    return subprocess.run(cmd, capture_output=True, text=True)
