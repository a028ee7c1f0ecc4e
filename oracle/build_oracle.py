"""Build recipes of the test oracle (test infrastructure only).

build_oracle(): compiles the C restatement b2sr_oracle.c into liboracle.so
    with gcc (OpenMP for the timed CPU baseline).
build_ref():    compiles the reference's own kernels, from the reference
    checkout's bmv_eval/backend/bsrbmv.cu (unmodified, reached through the
    include path), into oracle/_ref/bsrbmv_ref.cubin for sm_103a, and lists
    their mangled kernel names in oracle/_ref/kernels.txt (read with nm from a
    host-side object of the same translation unit).  Needs the reference
    checkout; a checkout-less machine uses the prebuilt files.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"
REF_CUBIN = REF_DIR / "bsrbmv_ref.cubin"
REF_NAMES = REF_DIR / "kernels.txt"
REFERENCE_BACKEND = Path(os.environ.get("B2SR_REFERENCE_ROOT", "/root/reference")) / "bmv_eval" / "backend"


def build_oracle(force: bool = False) -> Path:
    src = HERE / "b2sr_oracle.c"
    hdr = HERE / "b2sr_oracle.h"
    if (not force and ORACLE_LIB.exists()
            and ORACLE_LIB.stat().st_mtime >= max(src.stat().st_mtime, hdr.stat().st_mtime)):
        return ORACLE_LIB
    cc = os.environ.get("CC", "gcc")
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    subprocess.run([cc, "-O2", "-std=c99", "-fPIC", "-shared", "-fopenmp", str(src), "-o", str(tmp)],
                   check=True)
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def reference_present() -> bool:
    return (REFERENCE_BACKEND / "bsrbmv.cu").exists()


def build_ref(force: bool = False) -> Path | None:
    """Returns the cubin path, or None when neither the checkout nor a prebuilt cubin exists."""
    if not reference_present():
        return REF_CUBIN if REF_CUBIN.exists() and REF_NAMES.exists() else None
    if not force and REF_CUBIN.exists() and REF_NAMES.exists():
        return REF_CUBIN
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    REF_DIR.mkdir(exist_ok=True)
    wrapper = HERE / "ref_instantiate.cu"
    common = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w", "-I", str(REFERENCE_BACKEND)]
    subprocess.run([nvcc, *common, "-cubin", str(wrapper), "-o", str(REF_CUBIN)], check=True)
    obj = REF_DIR / "host_stubs.o"
    subprocess.run([nvcc, *common, "-c", str(wrapper), "-o", str(obj)], check=True)
    nm = subprocess.run(["nm", "--defined-only", str(obj)], check=True, capture_output=True, text=True)
    names = sorted({ln.split()[-1] for ln in nm.stdout.splitlines()
                    if any(k in ln for k in ("bmv", "ToBit")) and "__device_stub" not in ln
                    and ln.split()[-1].startswith("_Z") and "." not in ln.split()[-1]})
    obj.unlink()
    REF_NAMES.write_text("\n".join(names) + "\n")
    return REF_CUBIN


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
