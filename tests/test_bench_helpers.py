"""CPU tests of the benchmark's host-side helpers: the FP64 reference product
and error measures it reports, and the workload description both arms print."""
from __future__ import annotations

import importlib.util
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def load_bench():
    spec = importlib.util.spec_from_file_location("b2sr_bench", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_fp64_rows_matches_dense_product():
    bench = load_bench()
    rng = np.random.default_rng(0)
    d = (rng.random((50, 40)) < 0.1).astype(np.float64)
    d[7] = 0  # an empty row
    rowptr = np.concatenate([[0], np.cumsum(d.sum(1))]).astype(np.int32)
    colind = np.nonzero(d)[1].astype(np.int32)
    X = rng.standard_normal((40, 3))
    s, a = bench.fp64_rows(rowptr, colind, X)
    assert np.allclose(s, d @ X) and np.allclose(a, d @ np.abs(X))
    rows = np.array([3, 7, 49])
    s2, a2 = bench.fp64_rows(rowptr, colind, X[:, 0], rows)
    assert np.allclose(s2, (d @ X[:, 0])[rows]) and s2[1] == 0 and a2[1] == 0


def test_fp32_errors_flags():
    bench = load_bench()
    y64 = np.array([1.0, -2.0, 0.0, 1e-9])
    abs64 = np.array([1.0, 4.0, 0.0, 3.0])
    e = bench.fp32_errors(np.array([1.0, -2.0, 0.0, 0.0], np.float32), y64, abs64)
    assert e["within_bar"] and e["empty_rows_zero"]
    assert e["max_rel_err"] == 0.0  # the cancelling row (|y64| << its abs sum) is left to the row-abs measure
    assert 0 < e["max_err_rowabs"] < 1e-9
    bad = bench.fp32_errors(np.array([1.001, -2.0, 0.5, 0.0], np.float32), y64, abs64)
    assert not bad["within_bar"] and not bad["empty_rows_zero"]


def test_both_arms_describe_the_same_workload():
    bench = load_bench()
    rp = np.array([0, 1, 2], np.int32)
    ci = np.array([1, 0], np.int32)
    a = bench.workload_config(2, 2, bench.csr_sha256(rp, ci))
    b = bench.workload_config(2, 2, bench.csr_sha256(rp.copy(), ci.copy()))
    assert a == b and len(a["csr_sha256"]) == 64
    assert bench.csr_sha256(rp, ci[::-1].copy()) != a["csr_sha256"]
