"""The drop-in from C: tests/c_driver/drop_in_driver.c follows the reference's
test_bin_full_full / test_bin_bin_bin drivers with only their structure pass,
packer, vector packer and kernel launches replaced by libb2sr calls.  It is compiled with gcc against include/b2sr.h and the
built library, run at every tile size, and checks itself against host CSR
loops (exit status 0)."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "include" / "cuda_runtime.h").exists():
            return Path(cand)
    pytest.fail("CUDA toolkit headers not found")


@pytest.fixture(scope="module")
def driver(pkg, tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.fail("no C compiler")
    lib_dir = Path(pkg.library_path()).parent
    cuda = cuda_home()
    libdirs = [d for d in (cuda / "lib64", cuda / "lib", cuda / "targets" / "sbsa-linux" / "lib",
                           cuda / "targets" / "x86_64-linux" / "lib") if d.exists()]
    out = tmp_path_factory.mktemp("cdriver") / "drop_in_driver"
    cmd = [cc, "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", f"-I{cuda / 'include'}",
           str(ROOT / "tests" / "c_driver" / "drop_in_driver.c"), "-o", str(out)]
    for d in libdirs:
        cmd.append(f"-L{d}")
    cmd += ["-lcudart", f"-L{lib_dir}", "-lb2sr", f"-Wl,-rpath,{lib_dir}", "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return out


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_c_driver_through_the_shims_and_the_handle_api(driver, T):
    res = subprocess.run([str(driver), "20000", "16", str(T)], capture_output=True, text=True, timeout=300)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "PASSED" in res.stdout
