"""Benchmark of the B2SR binary SpMV hot path on one GB300.

Headline workload: R-MAT scale 20 (2^20 vertices, edge factor 16, a=0.57,
b=c=0.19, seed 1), symmetrised, de-duplicated, self-loops removed (seeded
synthetic data); bin_full_full SpMV y = A.x with x ~ U[0,1) FP32.  The tile
size is picked by a short timed sweep over T = 4/8/16/32 (all reported).

One step = one SpMV over the whole graph (the library's bin_full_full call),
timed with CUDA events on the launching stream.  L2 is flushed between steps,
outside the events, by reading a 256 MB buffer (a read leaves clean lines, so
the timed kernel pays no write-back of the flush).  `value` = GTEPS =
directed nnz per second / 1e9 with the inputs resident in HBM.  `roofline`
divides the algorithmic bytes by the dominant kernel's own time (events the
library records around it) and reads the ncu DRAM traffic from profiles/.
`e2e` runs the same call with each step's x copied from pinned host memory and
its y read back, double-buffered on copy streams (the serial figure is kept
beside it).  `accuracy` compares the headline y with an FP64 CSR product
computed here with numpy (max relative error per result, as the reference
drivers check every run, bmv_eval/test_bin_full_full.cu:355-370).  cuSPARSE,
the reference's own baseline, is called directly (cusparse_baseline.c:
cusparseSpMV with CUSPARSE_SPMV_CSR_ALG1 and ALG2, cusparseSpMM).  `extras`
hold the other workloads: the bit variants on the same graph, 32/64 frontiers
and SpMM k=64 on R-MAT scale 18, the 512-graph uneven batch replayed from a
CUDA graph, and 128-RHS forward+adjoint on scale 20, each next to cuSPARSE.

--impl reference times the reference's CPU path on the host cores: the
reference has no CPU SpMV, so its arm is the oracle's FP32 CSR SpMV (OpenMP
over rows) on the same graph, built by the oracle's own generator (the B2SR
library is not loaded in that arm).  Both arms print the same `config`,
including the SHA-256 of the CSR arrays.
"""
from __future__ import annotations

import argparse
import ctypes
import hashlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

RMAT = dict(scale=20, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1)
X_SEED = 2
L2_FLUSH_BYTES = 256 << 20


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profile(T: int):
    """Per-launch DRAM bytes of the main kernel from the committed ncu summary, if any."""
    p = ROOT / "profiles" / f"rowbin_spmv_kernel_rmat20_bin_full_full_T{T}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return int(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi SM clock / throttle-reason sampling while the timed loop runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, load_threshold_frac=0.0):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sms.append(float(parts[0]))
                maxs.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxs), "reasons": sorted(reasons),
                "samples": len(sms)}


def csr_sha256(rowptr, colind) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(rowptr, dtype=np.int32).tobytes())
    h.update(np.ascontiguousarray(colind, dtype=np.int32).tobytes())
    return h.hexdigest()


def workload_config(nrows, nnz, digest):
    """The `config` both arms print: the workload itself, nothing measured."""
    return {"workload": "rmat_s20_ef16_bin_full_full", "graph": "R-MAT", "scale": RMAT["scale"],
            "edge_factor": RMAT["edge_factor"], "abc": [RMAT["a"], RMAT["b"], RMAT["c"]], "seed": RMAT["seed"],
            "symmetrized": True, "self_loops": "removed", "duplicates": "removed", "nrows": nrows, "nnz": nnz,
            "variant": "bin_full_full", "x": f"U[0,1) FP32, numpy default_rng({X_SEED})", "csr_sha256": digest}


class CuSparse:
    """cusparse_baseline.c (built here with gcc, linked against libcusparse only)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            src = ROOT / "cusparse_baseline.c"
            out = ROOT / "_build" / "libcusparse_baseline.so"
            out.parent.mkdir(exist_ok=True)
            if not out.exists() or out.stat().st_mtime < src.stat().st_mtime:
                cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
                libdirs = [d for d in (cuda / "lib64", cuda / "targets" / "sbsa-linux" / "lib",
                                       cuda / "targets" / "x86_64-linux" / "lib") if d.exists()]
                cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-Wno-deprecated-declarations",
                       f"-I{cuda / 'include'}", str(src), "-o", str(out)]
                cmd += [f"-L{d}" for d in libdirs] + ["-lcusparse", "-lcudart"]
                subprocess.run(cmd, check=True, capture_output=True)
            lib = ctypes.CDLL(str(out))
            P = ctypes.c_void_p
            lib.cus_csr_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, ctypes.POINTER(P)]
            lib.cus_spmv.argtypes = [P, ctypes.c_int, P, P, ctypes.c_float, ctypes.c_int, P]
            lib.cus_spmm.argtypes = [P, ctypes.c_int, P, ctypes.c_int, P, ctypes.c_int, P]
            lib.cus_csr_destroy.argtypes = [P]
            lib.cus_csr_destroy.restype = None
            cls._lib = lib
        return cls._lib

    def __init__(self, torch, g, dev):
        self.rp = torch.from_numpy(g.rowptr).to(dev)
        self.ci = torch.from_numpy(g.colind).to(dev)
        self.h = ctypes.c_void_p()
        rc = self.lib().cus_csr_create(g.nrows, g.ncols, g.nnz, self.rp.data_ptr(), self.ci.data_ptr(),
                                       ctypes.byref(self.h))
        if rc != 0:
            raise RuntimeError(f"cus_csr_create failed ({rc})")

    def spmv(self, alg, x, y, stream, prepare=False):
        rc = self.lib().cus_spmv(self.h, alg, x.data_ptr(), y.data_ptr(), 0.0, int(prepare), stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"cus_spmv failed ({rc})")

    def spmm(self, transpose, X, Y, stream, prepare=False):
        rc = self.lib().cus_spmm(self.h, int(transpose), X.data_ptr(), X.shape[1], Y.data_ptr(), int(prepare),
                                 stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"cus_spmm failed ({rc})")

    def close(self):
        if self.h:
            self.lib().cus_csr_destroy(self.h)
            self.h = ctypes.c_void_p()


def fp64_rows(rowptr, colind, X, rows=None):
    """FP64 CSR product (values 1) for `rows` (all when None): X is [ncols] or
    [ncols, k]; returns (sum, sum of |terms|) per row."""
    rows = np.arange(rowptr.size - 1) if rows is None else np.asarray(rows)
    beg, end = rowptr[rows].astype(np.int64), rowptr[rows + 1].astype(np.int64)
    lens = end - beg
    idx = np.repeat(beg - np.concatenate([[0], np.cumsum(lens)[:-1]]), lens) + np.arange(lens.sum())
    vals = np.asarray(X, dtype=np.float64)[colind[idx]]
    shape = (rows.size,) + vals.shape[1:]
    s, a = np.zeros(shape), np.zeros(shape)
    nz = lens > 0
    starts = np.concatenate([[0], np.cumsum(lens)[:-1]])[nz]
    if vals.shape[0]:
        s[nz] = np.add.reduceat(vals, starts, axis=0)
        a[nz] = np.add.reduceat(np.abs(vals), starts, axis=0)
    return s, a


def fp32_errors(y, y64, abs64):
    """Error of an FP32 result against FP64.  The bar (the tests' bar) is
    |y - y64| <= 1e-5 * sum_j |A_ij x_j| per element, and empty rows exactly 0.
    Beside it, the plain element-wise relative error over the elements with
    |y64| >= 1e-3 of their row's absolute sum (where a sum cancels, FP32
    rounding of its terms alone exceeds 1e-5 of the small result)."""
    y = np.asarray(y, dtype=np.float64)
    d = np.abs(y - y64)
    keep = (abs64 > 0) & (np.abs(y64) >= 1e-3 * abs64)
    plain = float((d[keep] / np.abs(y64[keep])).max(initial=0.0))
    rowabs = float((d / np.maximum(abs64, 1e-30)).max(initial=0.0))
    zero_rows_exact = bool(np.all(y[abs64 == 0] == 0))
    return {"max_err_rowabs": rowabs, "max_rel_err": plain, "empty_rows_zero": zero_rows_exact,
            "within_bar": bool(rowabs <= 1e-5 and zero_rows_exact),
            "bar": "|y - y64| <= 1e-5 * sum_j |A_ij x_j|, empty rows 0"}


def make_graph(pkg):
    t0 = time.time()
    g = pkg.rmat(RMAT["scale"], RMAT["edge_factor"], RMAT["a"], RMAT["b"], RMAT["c"], RMAT["seed"])
    return g, time.time() - t0


def algorithmic_bytes(A, T: int) -> int:
    """bin_full_full: rowptr + colind + tiles read once, x read once, y written once."""
    w = T * (1 if T <= 8 else T // 8)
    return 4 * (A.nblockrows + 1) + A.nblocks * (4 + w) + 4 * A.ncols + 4 * A.nblockrows * T


def flush_l2(flush):
    """Evict L2 by reading a buffer twice its size (reads leave no dirty lines)."""
    flush.amax()


def max_over_ranks(torch, value, world, device):
    """The slowest rank's value (replicas run in lock step between barriers)."""
    if world <= 1:
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, ms_step, world):
    """Whole-job GTEPS of `world` replicas that each process units_per_rank per step."""
    return units_per_rank * world / (ms_step * 1e-3) / 1e9


def time_calls(torch, lib, fn, steps, warmup, flush, stream, kernel_timer=True):
    """Per-call CUDA-event times of fn() with L2 flushed before each call (outside
    the events), plus the library-recorded times of the dominant kernel of each call."""
    pkg_timer = sys.modules["bit_graphblas_gb300"].KernelTimer
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    launches = 0
    timer = pkg_timer(steps if kernel_timer else 0)
    with timer:
        for k in range(steps):
            if flush is not None:
                flush_l2(flush)
            evs[k][0].record(stream)
            fn()
            evs[k][1].record(stream)
            launches += lib.b2sr_last_launch_count()
        torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in evs]
    return ms, timer.ms, launches


def med(v):
    return statistics.median(v) if v else None


def rate(units, ms):
    return round(units / (ms * 1e-3) / 1e9, 3) if ms else None


def structure_bytes(A) -> int:
    w = A.tile_dim * (1 if A.tile_dim <= 8 else A.tile_dim // 8)
    return 4 * (A.nblockrows + 1) + A.nblocks * (4 + w)


def word_bytes(T: int) -> int:
    return 1 if T <= 8 else T // 8


def hbm_frac(nbytes, ms, peak):
    return round(nbytes / (ms * 1e-3) / 1e9 / peak, 4) if ms else None


def extra_s20_bits(torch, pkg, lib, g, mats, flush, stream, peak):
    """bin_bin_bin (frontier bits at 1% density, the BFS-step shape), bin_bin_full
    as int32 neighbour counts and as the reference's float counts, every tile size."""
    dev = flush.device
    f = torch.from_numpy((np.random.default_rng(3).random(g.ncols) < 0.01).astype(np.float32)).to(dev)
    out = {}
    for T, A in mats.items():
        xb = A.pack_bits(f, g.ncols)
        yb = torch.empty(A.nblockrows, dtype=pkg.word_dtype(T), device=dev)
        yc = torch.empty(A.padded_rows(), dtype=torch.int32, device=dev)
        yf = torch.empty(A.padded_rows(), dtype=torch.float32, device=dev)
        S = structure_bytes(A)
        vb = word_bytes(T)
        row = {}
        for name, variant, fn, nbytes in (
                ("bin_bin_bin", "bin_bin_bin", lambda: A.spmv_bin_bin_bin(xb, yb),
                 S + vb * (A.nblockcols + A.nblockrows)),
                ("bin_bin_count_i32", "bin_bin_count", lambda: A.spmv_bin_bin_count(xb, yc),
                 S + vb * A.nblockcols + 4 * A.padded_rows()),
                ("bin_bin_full_f32", "bin_bin_full", lambda: A.spmv_bin_bin_full(xb, yf),
                 S + vb * A.nblockcols + 4 * A.padded_rows())):
            ms, kms, _ = time_calls(torch, lib, fn, 30, 5, flush, stream)
            m, km = med(ms), med(kms)
            row[name] = {"ms": round(m, 5), "kernel_ms": round(km, 5) if km else None, "gteps": rate(g.nnz, m),
                         "algo_bytes": nbytes, "hbm_frac_call": hbm_frac(nbytes, m, peak),
                         "hbm_frac_kernel": hbm_frac(nbytes, km, peak), "algorithm": A.get_launch(variant)[3]}
        # exactness on the bench input: frontier count over each row's neighbours
        cs = np.concatenate([[0], np.cumsum(f.cpu().numpy()[g.colind].astype(np.int64))])
        want = cs[g.rowptr[1:]] - cs[g.rowptr[:-1]]
        row["counts_exact"] = bool(np.array_equal(yc[: g.nrows].cpu().numpy(), want))
        row["float_counts_exact"] = bool(np.array_equal(yf[: g.nrows].cpu().numpy(), want.astype(np.float32)))
        hit = np.zeros(A.padded_rows(), np.uint64)
        hit[: g.nrows] = want > 0
        words = (hit.reshape(-1, T) << np.arange(T - 1, -1, -1, dtype=np.uint64)).sum(axis=1)
        got = yb.cpu().numpy().view({4: np.uint8, 8: np.uint8, 16: np.uint16, 32: np.uint32}[T])
        row["bits_exact"] = bool(np.array_equal(got.astype(np.uint64), words))
        row["direction"] = bits_directions(torch, lib, A, g, f, flush, stream)
        out[str(T)] = row
    return out


def bits_directions(torch, lib, A, g, f, flush, stream):
    """bin_bin_bin and the masked BFS step (half the rows visited) under each
    direction, at the 1% frontier and at a 30% one; gteps counts every edge
    (the pull's work) so the rows compare directly.  exact: equal to the pull."""
    dev = flush.device
    A.transpose()  # built before the timed calls
    visited = A.pack_bits(torch.from_numpy((np.random.default_rng(8).random(A.padded_rows()) < 0.5)
                                           .astype(np.float32)).to(dev), A.padded_rows())
    dense = torch.from_numpy((np.random.default_rng(4).random(g.ncols) < 0.3).astype(np.float32)).to(dev)
    out = {}
    for label, frontier in (("d0.01", f), ("d0.30", dense)):
        xb = A.pack_bits(frontier, g.ncols)
        for step, call in (("bin_bin_bin", lambda y: A.spmv_bin_bin_bin(xb, y)),
                           ("masked", lambda y: A.spmv_bin_bin_bin_masked(xb, visited, y))):
            ref = None
            for direction in ("pull", "push", "auto"):
                A.set_launch("bin_bin_bin", direction=direction)
                y = torch.empty(A.nblockrows, dtype=xb.dtype, device=dev)
                ms, kms, _ = time_calls(torch, lib, lambda: call(y), 20, 5, flush, stream)
                m, km = med(ms), med(kms)
                if ref is None:
                    ref = y.clone()
                out[f"{label}_{step}_{direction}"] = {
                    "ms": round(m, 5), "kernel_ms": round(km, 5) if km else None, "gteps": rate(g.nnz, m),
                    "exact": bool(torch.equal(y, ref))}
                if label == "d0.01" and step == "bin_bin_bin":
                    # the same call replayed from a CUDA graph (no host launch gaps)
                    side = torch.cuda.Stream()
                    side.wait_stream(torch.cuda.current_stream())
                    with torch.cuda.stream(side):
                        call(y)  # scratch for the capture stream
                    torch.cuda.current_stream().wait_stream(side)
                    gr = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(gr, stream=side):
                        call(y)
                    ms, _, _ = time_calls(torch, lib, gr.replay, 20, 5, flush, stream, kernel_timer=False)
                    out[f"{label}_{step}_{direction}_graph"] = {"ms": round(med(ms), 5), "gteps": rate(g.nnz, med(ms)),
                                                                "exact": bool(torch.equal(y, ref))}
    # auto's time over the better forced direction's, per frontier and step
    out["auto_vs_best_forced"] = {
        f"{label}_{step}": round(out[f"{label}_{step}_auto"]["ms"]
                                 / min(out[f"{label}_{step}_pull"]["ms"], out[f"{label}_{step}_push"]["ms"]), 3)
        for label in ("d0.01", "d0.30") for step in ("bin_bin_bin", "masked")}
    A.set_launch("bin_bin_bin", direction="pull")
    return out


def extra_s18(torch, pkg, lib, flush, stream, peak):
    """R-MAT scale 18: 32 and 64 frontiers per vertex word (multi-source BFS
    shape) and FP32 SpMM with k = 64 (autotuned tile size)."""
    dev = flush.device
    g = pkg.rmat(18, 16, 0.57, 0.19, 0.19, 1)
    rng = np.random.default_rng(5)
    res = {"graph": {"scale": 18, "nrows": g.nrows, "nnz": g.nnz}}
    for bits in (32, 64):
        npdt = np.uint32 if bits == 32 else np.uint64
        dens = 10 ** rng.uniform(np.log10(0.001), np.log10(0.05), size=bits)
        X = np.zeros(g.ncols, npdt)
        for fr in range(bits):
            X |= (rng.random(g.ncols) < dens[fr]).astype(npdt) << npdt(fr)
        Xt = torch.from_numpy(X.view(np.int32 if bits == 32 else np.int64)).to(dev)
        sweep = {}
        for T in (4, 8, 16, 32):
            A = pkg.B2SRMatrix.from_graph(g, T, device=dev)
            Y = torch.empty(A.padded_rows(), dtype=Xt.dtype, device=dev)
            ms, kms, _ = time_calls(torch, lib, lambda: A.spmv_multi_bits(Xt, Y), 30, 5, flush, stream)
            nbytes = structure_bytes(A) + bits // 8 * (g.ncols + A.padded_rows())
            sweep[str(T)] = {"ms": round(med(ms), 5), "kernel_ms": round(med(kms), 5),
                             "gteps_frontier_edges": rate(g.nnz * bits, med(ms)), "algo_bytes": nbytes,
                             "hbm_frac_call": hbm_frac(nbytes, med(ms), peak),
                             "hbm_frac_kernel": hbm_frac(nbytes, med(kms), peak)}
            if T == 4:  # exactness on the bench input (OR over neighbours)
                rows = np.repeat(np.arange(g.nrows), np.diff(g.rowptr))
                want = np.zeros(g.nrows, npdt)
                np.bitwise_or.at(want, rows, X[g.colind])
                sweep[str(T)]["exact"] = bool(np.array_equal(Y[: g.nrows].cpu().numpy().view(npdt), want))
            A.close()
        best = min(sweep, key=lambda t: sweep[t]["ms"])
        res[f"multi_bits_{bits}"] = {"best_tile": int(best), "sweep": sweep}
    # FP32 SpMM, k = 64, tile size and launch picked by the library's autotuner
    k = 64
    Xd = torch.from_numpy(np.random.default_rng(6).standard_normal((g.ncols, k), dtype=np.float32)).to(dev)
    t0 = time.time()
    A, info = pkg.B2SRMatrix.autotuned(g, "bin_full_full", k=k, device=dev)
    tune_s = time.time() - t0
    Y = torch.empty(A.padded_rows(), k, device=dev)
    ms, kms, _ = time_calls(torch, lib, lambda: A.spmm(Xd, Y), 20, 5, flush, stream)
    nbytes = structure_bytes(A) + 4 * k * (g.ncols + A.padded_rows())
    spmm = {"tile_dim": A.tile_dim, "autotune": {kk: (round(v, 5) if isinstance(v, float) else v)
                                                  for kk, v in info.items()}, "autotune_s": round(tune_s, 2),
            "ms": round(med(ms), 5), "kernel_ms": round(med(kms), 5), "gteps_rhs_edges": rate(g.nnz * k, med(ms)),
            "algo_bytes": nbytes, "hbm_frac_call": hbm_frac(nbytes, med(ms), peak)}
    spmm["accuracy_vs_fp64"] = sampled_errors(g, Xd, Y)
    spmm["cusparse_spmm"] = cusparse_spmm(torch, g, Xd, Y[: g.nrows], flush, stream)
    res["spmm_k64"] = spmm
    A.close()
    # the same SpMM at every tile size: the row-task kernel (the default) and
    # the merge-path kernel (launch option algorithm = merge)
    tiles = {}
    for T in (4, 8, 16, 32):
        A = pkg.B2SRMatrix.from_graph(g, T, device=dev)
        Y = torch.empty(A.padded_rows(), k, device=dev)
        row = {}
        for algo in ("auto", "merge"):
            A.set_launch("bin_full_full", algorithm=algo)
            ms, kms, _ = time_calls(torch, lib, lambda: A.spmm(Xd, Y), 10, 3, flush, stream)
            name = "rows" if algo == "auto" else "merge"
            row[name + "_ms"] = round(med(ms), 5)
            e = sampled_errors(g, Xd, Y)
            row[name + "_max_err_rowabs"] = e["max_err_rowabs"]
            row[name + "_within_bar"] = e["within_bar"]
        tiles[str(T)] = row
        A.close()
    res["spmm_k64_tiles"] = tiles
    return res


def cusparse_spmm(torch, g, X, Y_ours, flush, stream, steps=20, transpose=False):
    """cusparseSpMM (CSR, FP32, CUSPARSE_SPMM_CSR_ALG2) of the same graph and X,
    timed like ours, and its largest difference from our result."""
    try:
        dev = X.device
        cs = CuSparse(torch, g, dev)
        Yc = torch.empty(g.ncols if transpose else g.nrows, X.shape[1], device=dev)
        cs.spmm(transpose, X, Yc, stream, prepare=True)
        torch.cuda.synchronize()
        lib = sys.modules["bit_graphblas_gb300"]._lib.load()
        ms, _, _ = time_calls(torch, lib, lambda: cs.spmm(transpose, X, Yc, stream), steps, 3, flush, stream,
                              kernel_timer=False)
        cm = med(ms)
        diff = float((Yc - Y_ours).abs().max() / Yc.abs().max().clamp_min(1e-30))
        cs.close()
        # cuSPARSE's own FP32 error on the same sampled rows (A is symmetric,
        # so the rows of A^T are the rows of A), for scale
        acc = sampled_errors(g, X, Yc)
        return {"ms": round(cm, 5), "gteps_rhs_edges": rate(g.nnz * X.shape[1], cm), "max_rel_diff_vs_b2sr": diff,
                "accuracy_vs_fp64": acc,
                "api": "cusparseSpMM(CSR, FP32, CUSPARSE_SPMM_CSR_ALG2" + (", A^T)" if transpose else ")")}
    except Exception as e:  # pragma: no cover - reported, not fatal
        return {"error": repr(e)[:200]}


def sampled_errors(g, X, Y, nsample=4096, seed=11):
    """fp32_errors of Y's rows against FP64 on a seeded sample of rows."""
    rows = np.sort(np.random.default_rng(seed).choice(g.nrows, size=min(nsample, g.nrows), replace=False))
    y64, a64 = fp64_rows(g.rowptr, g.colind, X.cpu().numpy(), rows)
    import torch
    e = fp32_errors(Y[torch.from_numpy(rows).to(Y.device)].cpu().numpy(), y64, a64)
    e["rows_checked"] = int(rows.size)
    return e




def extra_batch512(torch, pkg, lib, flush, stream, peak):
    """512 Erdos-Renyi graphs (n log-uniform in 64..65536, degree U[4, 32]) stacked
    block-diagonally in one B2SR, FP32 features of width 64: one persistent SpMM
    launch (device work queue over merge-path chunks of tile-rows) replayed from a
    captured CUDA graph."""
    dev = flush.device
    t0 = time.time()
    g, offsets, sizes, degrees = pkg.er_batch(512, 64, 65536, 4, 32, align=32, seed=4)
    gen_s = time.time() - t0
    k = 64
    X = torch.from_numpy(np.random.default_rng(7).standard_normal((g.ncols, k), dtype=np.float32)).to(dev)
    A, info = pkg.B2SRMatrix.autotuned(g, "bin_full_full", k=k, device=dev)
    Y = torch.empty(A.padded_rows(), k, device=dev)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(3):
            A.spmm(X, Y)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        A.spmm(X, Y)
    ms_graph, _, _ = time_calls(torch, lib, graph.replay, 20, 3, flush, stream, kernel_timer=False)
    ms_call, kms, launches = time_calls(torch, lib, lambda: A.spmm(X, Y), 20, 3, flush, stream)
    # exactness of the graph replay against the direct call
    Yg = Y.clone()
    graph.replay()
    torch.cuda.synchronize()
    nbytes = structure_bytes(A) + 4 * k * (g.ncols + A.padded_rows())
    res = {"graphs": 512, "nrows": g.nrows, "nnz": g.nnz, "tile_dim": A.tile_dim, "gen_s": round(gen_s, 2),
           "smallest": int(sizes.min()), "largest": int(sizes.max()),
           "ms_graph_replay": round(med(ms_graph), 5), "ms_direct_call": round(med(ms_call), 5),
           "kernel_ms": round(med(kms), 5), "launches_per_call": launches // 20,
           "gteps_rhs_edges": rate(g.nnz * k, med(ms_graph)), "algo_bytes": nbytes,
           "hbm_frac": hbm_frac(nbytes, med(ms_graph), peak), "replay_equals_call": bool(torch.equal(Yg, Y)),
           "autotune": {kk: (round(v, 5) if isinstance(v, float) else v) for kk, v in info.items()}}
    res["accuracy_vs_fp64"] = sampled_errors(g, X, Y)
    res["cusparse_spmm"] = cusparse_spmm(torch, g, X, Y[: g.nrows], flush, stream, steps=10)
    A.close()
    return res


def extra_rhs128(torch, pkg, lib, g, flush, stream, peak):
    """R-MAT scale 20, 128 right-hand sides: batched forward Y = A.X plus adjoint
    dX = A^T.dY (two SpMM launches over A and the transposed B2SR) against 128
    plain single-vector forward and 128 adjoint launches; then the autograd path
    and a 2-layer sum-aggregation GNN step (hidden 128)."""
    dev = flush.device
    k = 128
    rng = np.random.default_rng(8)
    X = torch.from_numpy(rng.standard_normal((g.ncols, k), dtype=np.float32)).to(dev)
    t0 = time.time()
    A, info = pkg.B2SRMatrix.autotuned(g, "bin_full_full", k=k, device=dev)
    tune_s = time.time() - t0
    t0 = time.time()
    At = A.transpose()
    torch.cuda.synchronize()
    transpose_s = time.time() - t0
    dY = torch.from_numpy(rng.standard_normal((At.ncols, k), dtype=np.float32)).to(dev)  # padded rows of A
    dY[g.nrows:] = 0
    Y = torch.empty(A.padded_rows(), k, device=dev)
    dX = torch.empty(At.padded_rows(), k, device=dev)

    def batched():
        A.spmm(X, Y)
        At.spmm(dY, dX)

    ms_b, kms_b, l_b = time_calls(torch, lib, batched, 5, 3, flush, stream)
    A.spmm(X, Y)
    At.spmm(dY, dX)
    torch.cuda.synchronize()
    # A is symmetric (symmetrised R-MAT): row j of A^T is row j of A
    acc_fwd = sampled_errors(g, X, Y)
    acc_adj = sampled_errors(g, dY, dX)
    cus_fwd = cusparse_spmm(torch, g, X, Y[: g.nrows], flush, stream, steps=5)
    cus_adj = cusparse_spmm(torch, g, dY[: g.nrows], dX[: g.ncols], flush, stream, steps=5, transpose=True)
    Xt = X.t().contiguous()            # 128 plain vectors, contiguous each
    dYt = dY.t().contiguous()
    y1 = torch.empty(k, A.padded_rows(), device=dev)
    dx1 = torch.empty(k, At.padded_rows(), device=dev)
    A.spmv_bin_full_full(Xt[0], y1[0])
    At.spmv_bin_full_full(dYt[0], dx1[0])

    def plain():
        for i in range(k):
            A.spmv_bin_full_full(Xt[i], y1[i])
        for i in range(k):
            At.spmv_bin_full_full(dYt[i], dx1[i])

    ms_p, _, _ = time_calls(torch, lib, plain, 3, 1, flush, stream, kernel_timer=False)
    # the two must agree (same sums, different summation grouping)
    scale = float(Y[: g.nrows].abs().max())
    fwd_diff = float((y1.t()[: g.nrows] - Y[: g.nrows]).abs().max()) / scale
    adj_diff = float((dx1.t()[: g.ncols] - dX[: g.ncols]).abs().max()) / float(dX[: g.ncols].abs().max())

    # autograd path (torch.autograd.Function over the C ABI), fwd + bwd
    Xg = X.detach().clone().requires_grad_(True)
    dYg = dY[: g.nrows]

    def autograd_step():
        Xg.grad = None
        out = pkg.aggregate(A, Xg)
        out.backward(dYg)

    ms_ag, _, _ = time_calls(torch, lib, autograd_step, 5, 2, flush, stream, kernel_timer=False)
    # 2-layer GNN step (forward + backward), hidden 128, random-init FP32 weights
    gen = torch.Generator().manual_seed(9)
    net = pkg.SumAggGNN(k, 128, 128, generator=gen, device=dev)
    Xn = X[: g.ncols]

    def gnn_step():
        net.zero_grad(set_to_none=True)
        out = net(A, Xn)
        out.backward(dYg)

    ms_gnn, _, _ = time_calls(torch, lib, gnn_step, 5, 2, flush, stream, kernel_timer=False)
    S = structure_bytes(A) + structure_bytes(At)
    nbytes = S + 4 * k * 2 * (A.padded_rows() + At.padded_rows())
    res = {"k": k, "tile_dim": A.tile_dim, "autotune_s": round(tune_s, 2), "transpose_s": round(transpose_s, 3),
           "batched_fwd_adj_ms": round(med(ms_b), 4), "batched_kernel_ms_each": [round(v, 4) for v in kms_b[:4]],
           "plain_256_spmv_ms": round(med(ms_p), 4),
           "speedup_batched_vs_plain": round(med(ms_p) / med(ms_b), 2),
           "gteps_batched": rate(2 * g.nnz * k, med(ms_b)), "gteps_plain": rate(2 * g.nnz * k, med(ms_p)),
           "algo_bytes_batched": nbytes, "hbm_frac_batched": hbm_frac(nbytes, med(ms_b), peak),
           "max_rel_diff_plain_vs_batched": {"forward": fwd_diff, "adjoint": adj_diff},
           "accuracy_vs_fp64": {"forward": acc_fwd, "adjoint": acc_adj},
           "cusparse_spmm_forward": cus_fwd, "cusparse_spmm_adjoint": cus_adj,
           "autograd_fwd_bwd_ms": round(med(ms_ag), 4), "gnn2_step_ms": round(med(ms_gnn), 4),
           "launches_batched": l_b // 5}
    At.close()
    A.close()
    return res


def e2e_serial(torch, A, x_np, y, stream, steps, warmup):
    """ms per step of H2D x, SpMV, D2H y, back to back on one stream."""
    x_host = torch.from_numpy(x_np).pin_memory()
    y_host = torch.empty(A.padded_rows(), dtype=torch.float32).pin_memory()
    xd = torch.empty(x_np.size, dtype=torch.float32, device=y.device)
    for _ in range(warmup):
        xd.copy_(x_host, non_blocking=True)
        A.spmv_bin_full_full(xd, y)
        y_host.copy_(y, non_blocking=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        xd.copy_(x_host, non_blocking=True)
        A.spmv_bin_full_full(xd, y)
        y_host.copy_(y, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def e2e_pipelined(torch, A, x_np, stream, steps, warmup):
    """ms per step with every step's H2D copy of x and D2H copy of y, double
    buffered: copies run on their own streams, ordered by events against the
    multiply that uses the same buffer."""
    dev = torch.device("cuda", torch.cuda.current_device())
    xh = [torch.from_numpy(x_np).pin_memory() for _ in range(2)]
    yh = [torch.empty(A.padded_rows(), dtype=torch.float32).pin_memory() for _ in range(2)]
    xd = [torch.empty(x_np.size, dtype=torch.float32, device=dev) for _ in range(2)]
    yd = [torch.empty(A.padded_rows(), dtype=torch.float32, device=dev) for _ in range(2)]
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_mul = [torch.cuda.Event() for _ in range(2)]
    ev_out = [torch.cuda.Event() for _ in range(2)]

    def step(i):
        b = i & 1
        s_in.wait_event(ev_mul[b])       # the multiply that last read xd[b] is done
        with torch.cuda.stream(s_in):
            xd[b].copy_(xh[b], non_blocking=True)
        ev_in[b].record(s_in)
        stream.wait_event(ev_in[b])
        stream.wait_event(ev_out[b])     # the copy that last read yd[b] is done
        A.spmv_bin_full_full(xd[b], yd[b])
        ev_mul[b].record(stream)
        s_out.wait_event(ev_mul[b])
        with torch.cuda.stream(s_out):
            yh[b].copy_(yd[b], non_blocking=True)
        ev_out[b].record(s_out)

    for i in range(warmup):
        step(i)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s_in.wait_stream(stream)
    for i in range(steps):
        step(i)
    stream.wait_stream(s_in)
    stream.wait_stream(s_out)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def run_ours(args):
    import torch
    import __graft_entry__ as entry

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pkg = entry.load_package()
    lib = pkg._lib.load()

    g, gen_s = make_graph(pkg)
    digest = csr_sha256(g.rowptr, g.colind)
    rng = np.random.default_rng(X_SEED)
    x_np = rng.random(g.ncols, dtype=np.float32)
    x = torch.from_numpy(x_np).to(dev)
    flush = torch.ones(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    peak, peak_kind = load_peaks()

    # tile-size sweep (part of the autotuning; every size reported)
    tiles = [int(t) for t in args.tiles.split(",")]
    sweep = {}
    mats = {}
    for T in tiles:
        t0 = time.time()
        A = pkg.B2SRMatrix.from_graph(g, T, device=dev)
        torch.cuda.synchronize()
        pack_s = time.time() - t0
        if args.algorithm != "auto" or args.gather != "auto":
            A.set_launch("bin_full_full", algorithm=args.algorithm, gather=args.gather)
        y = torch.empty(A.padded_rows(), device=dev)
        ms, kms, _ = time_calls(torch, lib, lambda: A.spmv_bin_full_full(x, y), 20, 5, flush, stream)
        sweep[T] = {"ms": round(med(ms), 5), "kernel_ms": round(med(kms), 5), "nblocks": A.nblocks,
                    "pack_s": round(pack_s, 3), "algo_bytes": algorithmic_bytes(A, T),
                    "hbm_frac_kernel": hbm_frac(algorithmic_bytes(A, T), med(kms), peak)}
        mats[T] = A
    T = min(sweep, key=lambda t: sweep[t]["ms"]) if args.tile == 0 else args.tile
    A = mats[T]
    y = torch.empty(A.padded_rows(), device=dev)

    # correctness gate on the bench workload itself (FP64 CSR oracle is test infra;
    # here a size-independent property: x = 1 gives the exact degrees)
    ones = torch.ones(g.ncols, device=dev)
    deg = A.spmv_bin_full_full(ones)[: g.nrows].cpu().numpy()
    assert np.array_equal(deg, np.diff(g.rowptr).astype(np.float32)), "degree check failed"

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_wall = time.time()
        ms, _, launches = time_calls(torch, lib, lambda: A.spmv_bin_full_full(x, y), args.steps, args.warmup,
                                     flush, stream, kernel_timer=False)
        t_wall = time.time() - t_wall
    torch.cuda.synchronize()
    # the dominant kernel's own time for the roofline: a second pass with the
    # library's kernel timer armed (its events sit between the kernels, so the
    # step time above is taken without them)
    _, kms, _ = time_calls(torch, lib, lambda: A.spmv_bin_full_full(x, y), args.steps, 2, flush, stream)
    if world > 1:
        torch.distributed.barrier()
    clocks = clk.summary()
    ms_step = max_over_ranks(torch, sum(ms) / len(ms), world, dev)
    kernel_ms = sum(kms) / len(kms) if kms else None
    nnz = g.nnz
    gteps = replica_throughput(nnz, ms_step, world)

    # e2e: public API with host buffers, copies inside the timed region
    e2e_steps = min(args.steps, 500)
    e2e_serial_ms = e2e_serial(torch, A, x_np, y, stream, e2e_steps, max(args.warmup, 3))
    e2e_ms = e2e_pipelined(torch, A, x_np, stream, e2e_steps, max(args.warmup, 3))
    e2e = {"value": round(nnz / (e2e_ms * 1e-3) / 1e9 * world, 3), "unit": "GTEPS",
           "ms_per_step": round(e2e_ms, 5), "h2d_bytes_per_step": int(g.ncols * 4),
           "d2h_bytes_per_step": int(A.padded_rows() * 4), "steps": e2e_steps,
           "note": "every step copies its x from pinned host memory and reads its y back; two buffers and "
                   "two copy streams let step i's copies overlap the neighbouring steps' multiplies; L2 not flushed",
           "serial": {"value": round(nnz / (e2e_serial_ms * 1e-3) / 1e9 * world, 3),
                      "ms_per_step": round(e2e_serial_ms, 5),
                      "note": "H2D, SpMV, D2H back to back on one stream"}}

    # accuracy of the headline result: the y of the last timed call against an
    # FP64 CSR product of the same graph and x (numpy, here)
    y64, abs64 = fp64_rows(g.rowptr, g.colind, x_np)
    accuracy = {"bin_full_full": fp32_errors(y[: g.nrows].cpu().numpy(), y64, abs64),
                "reference": "FP64 CSR SpMV of the same graph and x (numpy)",
                "padding_rows_zero": bool(torch.all(y[g.nrows:] == 0).item())}

    # cuSPARSE CSR SpMV (the reference's own baseline) on the same graph and GPU:
    # cusparseSpMV with an explicit CSR algorithm, values 1, y = A.x
    cus = {}
    try:
        cs = CuSparse(torch, g, dev)
        yc = torch.empty(g.nrows, device=dev)
        for alg, name in ((1, "CUSPARSE_SPMV_CSR_ALG1"), (2, "CUSPARSE_SPMV_CSR_ALG2")):
            cs.spmv(alg, x, yc, stream, prepare=True)
            cms, _, _ = time_calls(torch, lib, lambda: cs.spmv(alg, x, yc, stream), 50, 5, flush, stream,
                                   kernel_timer=False)
            cm = med(cms)
            cus[name] = {"ms": round(cm, 5), "gteps": round(nnz / (cm * 1e-3) / 1e9, 3),
                         "bytes": 4 * (g.nrows + 1) + 8 * nnz + 4 * g.ncols + 4 * g.nrows,
                         "b2sr_speedup": round(cm / ms_step, 3),
                         "accuracy_vs_fp64": fp32_errors(yc.cpu().numpy(), y64, abs64),
                         "api": f"cusparseSpMV(CSR, FP32, {name})"}
        cs.close()
    except Exception as e:  # pragma: no cover - reported, not fatal
        cus = {"error": repr(e)[:200]}

    algo = algorithmic_bytes(A, T)
    achieved = algo / (kernel_ms * 1e-3) / 1e9 if kernel_ms else algo / (ms_step * 1e-3) / 1e9
    traffic = traffic_from_profile(T)
    kernel_name = {"rowbin": "rowbin_spmv_kernel", "merge": "merge_spmv_kernel"}.get(
        A.get_launch("bin_full_full")[3], "rowbin_spmv_kernel")
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s",
                "algorithmic_bytes_per_launch": algo, "kernel": kernel_name,
                "kernel_ms": round(kernel_ms, 5) if kernel_ms else None,
                "timed": "dominant kernel per call, CUDA events recorded by the library on the launching stream "
                         "(a second pass of the same steps; the step time is taken without these events)",
                "achieved_whole_call": round(algo / (ms_step * 1e-3) / 1e9, 1),
                "frac_whole_call": round(algo / (ms_step * 1e-3) / 1e9 / peak, 4)}

    extras = {}
    if not args.no_extras:
        wanted = set(args.extras.split(","))
        for key, name, fn in (
                ("bits", "rmat20_bits_variants", lambda: extra_s20_bits(torch, pkg, lib, g, mats, flush, stream, peak)),
                ("multi", "rmat18_multi_rhs", lambda: extra_s18(torch, pkg, lib, flush, stream, peak)),
                ("batch", "uneven_batch_512", lambda: extra_batch512(torch, pkg, lib, flush, stream, peak)),
                ("rhs128", "rmat20_rhs128_fwd_adjoint", lambda: extra_rhs128(torch, pkg, lib, g, flush, stream, peak))):
            if "all" not in wanted and key not in wanted:
                continue
            t0 = time.time()
            try:
                extras[name] = fn()
            except Exception as e:  # reported, not fatal to the headline
                extras[name] = {"error": repr(e)[:300]}
            extras[name]["wall_s"] = round(time.time() - t0, 1)
            torch.cuda.empty_cache()
    for t, m in mats.items():
        if t != T:
            m.close()

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(g, x_np, budget_s=args.cpu_seconds)

    line = {
        "metric": "B2SR SpMV GTEPS (bin_full_full, single vector)",
        "value": round(gteps, 3), "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded R-MAT)",
        "config": workload_config(g.nrows, nnz, digest),
        "setup": {"tile_dim": T, "nblocks": A.nblocks,
                  "l2": "flushed between steps (256 MB read, outside the timed events)",
                  "parallelism": "replicas" if world > 1 else "single GPU",
                  "tile_sweep": {str(k): v for k, v in sweep.items()},
                  "launch": dict(zip(("threads", "items_per_thread", "ctas_per_sm", "algorithm", "gather",
                                      "rhs_block", "direction"), A.get_launch("bin_full_full"))),
                  "graph_gen_s": round(gen_s, 2)},
        "accuracy": accuracy,
        "roofline": roofline,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "baselines": {"cusparse_csr_spmv_fp32": cus},
        "wall_s_timed_loop": round(t_wall, 3),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    line["extras"] = extras  # last: the long part of the line
    if rank == 0:
        print(json.dumps(line), flush=True)
    A.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline(g, x_np, budget_s=10.0, sample_rows=None):
    """The oracle's FP32 CSR SpMV (OpenMP, all host threads) on the host cores."""
    import __graft_entry__ as entry

    orc = entry.load_oracle()
    rp, ci = g.rowptr, g.colind
    nrows = g.nrows if sample_rows is None else min(sample_rows, g.nrows)
    rp_s = rp[: nrows + 1]
    y = np.zeros(nrows, np.float32)
    orc.csr_spmv_f32_omp(rp_s, ci, nrows, x_np, y)  # warm-up
    reps, t0 = 0, time.perf_counter()
    used = 1
    while True:
        _, used = orc.csr_spmv_f32_omp(rp_s, ci, nrows, x_np, y)
        reps += 1
        el = time.perf_counter() - t0
        if (el >= budget_s and reps >= 3) or reps >= 1000:
            break
    per = el / reps
    nnz = int(rp_s[-1])
    return {"value": round(nnz / per / 1e9, 4), "unit": "GTEPS", "cores": int(used), "kind": "port",
            "ms_per_spmv": round(per * 1e3, 3),
            "sample": f"{nrows} of {g.nrows} rows ({nnz} nnz) of the R-MAT s20 graph, "
                      f"{reps} full passes in {el:.1f}s; FP32 CSR, OpenMP static over rows"}


def run_reference(args):
    """The reference's CPU path on the host cores.  The reference has no CPU
    SpMV, so this times the oracle's FP32 CSR SpMV (OpenMP over rows, every
    host thread) on the headline graph, built by the oracle's own R-MAT
    generator: the B2SR library is not loaded here."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import __graft_entry__ as entry

    orc = entry.load_oracle()
    rowptr, colind = orc.rmat_csr(RMAT["scale"], RMAT["edge_factor"], RMAT["a"], RMAT["b"], RMAT["c"],
                                  RMAT["seed"])
    nrows, nnz_all = rowptr.size - 1, int(rowptr[-1])
    digest = csr_sha256(rowptr, colind)
    x_np = np.random.default_rng(X_SEED).random(nrows, dtype=np.float32)
    # bound the sample so that W + K steps stay within ~2 minutes
    y = np.zeros(nrows, np.float32)
    t0 = time.perf_counter()
    _, used = orc.csr_spmv_f32_omp(rowptr, colind, nrows, x_np, y)
    t_full = time.perf_counter() - t0
    budget = 120.0
    frac = min(1.0, budget / max(t_full * (args.steps + args.warmup), 1e-9))
    rows = max(1, int(nrows * frac))
    rp_s = rowptr[: rows + 1]
    ys = np.zeros(rows, np.float32)
    for _ in range(args.warmup):
        orc.csr_spmv_f32_omp(rp_s, colind, rows, x_np, ys)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        orc.csr_spmv_f32_omp(rp_s, colind, rows, x_np, ys)
        times.append(time.perf_counter() - t0)
    per = sum(times) / len(times)
    nnz = int(rp_s[-1])
    val = nnz / per / 1e9
    sample = (f"rows [0, {rows}) of {nrows} ({nnz} of {nnz_all} nnz, fraction {nnz / max(nnz_all, 1):.4f}) per "
              f"step; the reference has no CPU SpMV, so this is the oracle's FP32 CSR SpMV (OpenMP, static "
              f"schedule over rows)")
    line = {
        "impl": "reference",
        "metric": "B2SR SpMV GTEPS (bin_full_full, single vector)",
        "value": round(val, 4), "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(per * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded R-MAT)",
        "config": workload_config(nrows, nnz_all, digest),
        "cpu_baseline": {"value": round(val, 4), "unit": "GTEPS", "cores": int(used), "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(val, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--tile", type=int, default=0, help="0 = pick by the timed sweep")
    ap.add_argument("--algorithm", default="auto", choices=["auto", "merge", "rowbin"],
                    help="bin_full_full kernel family (launch option; default: the library's choice)")
    ap.add_argument("--gather", default="auto", choices=["auto", "ldg", "texture", "sparse"],
                    help="row-binned x gather path (launch option; default: the library's choice)")
    ap.add_argument("--tiles", default="4,8,16,32")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the other workloads (bit variants, multi-RHS, uneven batch, 128-RHS adjoint)")
    ap.add_argument("--extras", default="all",
                    help="comma list of the other workloads to run: bits, multi, batch, rhs128 (default all)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        import __graft_entry__ as entry
        entry.build()
        run_ours(args)


if __name__ == "__main__":
    main()
