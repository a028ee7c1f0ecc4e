"""The reference's own drivers, bmv_eval/test_bin_full_full.cu and
test_bin_bin_bin.cu, relinked against libb2sr: oracle/ref_drivers.py copies
them from the reference checkout with only their structure pass, packer,
vector packer and timed kernel launches bound to the C ABI (plus a dump of x
and y), and this test builds them in timing mode for sm_103a at every tile
size, runs them on a Matrix Market file written from a seeded graph, and
checks the dumped y against the oracle.  The drivers draw their own x
(srand(time(0))) and launch TEST_TIMES = 5 accumulating multiplies, so y is
5 A.x (exact: x is 0/1) for bin_full_full and the OR product for
bin_bin_bin."""
from __future__ import annotations

import importlib.util
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
TILES = (4, 8, 16, 32)
TEST_TIMES = 5  # the drivers' #define


def ref_drivers():
    spec = importlib.util.spec_from_file_location("b2sr_ref_drivers", ROOT / "oracle" / "ref_drivers.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def built_drivers(pkg, tmp_path_factory):
    rd = ref_drivers()
    if rd.prepare() is None:
        pytest.skip("the patched reference drivers were not prepared (no reference checkout where build() ran)")
    out = tmp_path_factory.mktemp("refdrivers")
    lib_dir = Path(pkg.library_path()).parent
    jobs = [(name, T) for name in rd.DRIVERS for T in TILES]

    def build(job):
        name, T = job
        exe = out / f"{name[:-3]}_T{T}"
        return job, exe, rd.compile_driver(name, T, lib_dir, ROOT / "include", exe)

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(build, jobs))
    exes = {}
    for job, exe, res in results:
        assert res.returncode == 0, f"{job}: {res.stderr[-3000:]}"
        exes[job] = exe
    return exes


@pytest.fixture(scope="module")
def mtx_graph(pkg, tmp_path_factory):
    """R-MAT scale 12 (hub rows spanning many tiles) as a symmetric pattern
    Matrix Market file, each undirected edge once (lower triangle)."""
    g = pkg.rmat(12, 16, seed=51)
    rows = np.repeat(np.arange(g.nrows), np.diff(g.rowptr))
    low = rows > g.colind
    path = tmp_path_factory.mktemp("mtx") / "rmat12.mtx"
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern symmetric\n")
        f.write(f"{g.nrows} {g.ncols} {int(low.sum())}\n")
        np.savetxt(f, np.stack([rows[low] + 1, g.colind[low] + 1], 1), fmt="%d")
    return g, path


def run_driver(exe, mtx, dump):
    env = dict(os.environ, B2SR_DUMP=str(dump))
    res = subprocess.run([str(exe), str(mtx), "0"], capture_output=True, text=True, timeout=300, env=env)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    raw = dump.read_bytes()
    nrows, nb, T = (int(v) for v in np.frombuffer(raw[:12], np.int32))
    x = np.frombuffer(raw[12:12 + 4 * nrows], np.float32)
    return nrows, nb, T, x, raw[12 + 4 * nrows:], res.stdout


@pytest.mark.parametrize("T", TILES)
def test_reference_bin_full_full_driver_relinked(orc, built_drivers, mtx_graph, tmp_path, T):
    g, mtx = mtx_graph
    nrows, nb, t, x, ybytes, out = run_driver(built_drivers[("test_bin_full_full.cu", T)], mtx, tmp_path / "y.bin")
    assert (nrows, t) == (g.nrows, T) and set(np.unique(x)) <= {0.0, 1.0}
    y = np.frombuffer(ybytes, np.float32)
    assert y.size == nb * T
    want = TEST_TIMES * orc.csr_spmv_count(g.rowptr, g.colind, g.nrows, x > 0)
    assert np.array_equal(y[:nrows], want.astype(np.float32)), "bin_full_full y differs from the oracle"
    assert not np.any(y[nrows:])
    print(f"T={T}: relinked reference driver printed {out.strip()!r} (ms per launch)")


@pytest.mark.parametrize("T", TILES)
def test_reference_bin_bin_bin_driver_relinked(orc, built_drivers, mtx_graph, tmp_path, T):
    g, mtx = mtx_graph
    nrows, nb, t, x, ybytes, out = run_driver(built_drivers[("test_bin_bin_bin.cu", T)], mtx, tmp_path / "y.bin")
    assert (nrows, t) == (g.nrows, T)
    y = np.frombuffer(ybytes, {4: np.uint8, 8: np.uint8, 16: np.uint16, 32: np.uint32}[T])
    brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
    want = orc.bmv_bin_bin_bin(T, brp, bci, tiles, orc.pack_vec_bits(x, T))
    assert np.array_equal(y[:nb], want), "bin_bin_bin y differs from the oracle"
    print(f"T={T}: relinked reference driver printed {out.strip()!r} (ms per launch)")
