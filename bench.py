"""Benchmark of the B2SR binary SpMV hot path on one GB300.

Workload (the spec configuration): R-MAT scale 20 (2^20 vertices, edge
factor 16, a=0.57, b=c=0.19), symmetrised, de-duplicated, self-loops removed,
seeded synthetic data; bin_full_full SpMV y = A.x with x ~ U[0,1) FP32.  The
tile size is picked by a short timed sweep over T = 4/8/16/32 (all reported).

One step = one SpMV over the whole graph (the library's bin_full_full call),
timed with CUDA events on the launching stream; L2 is flushed between steps,
outside the timed events, by reading a 256 MB buffer (a read leaves clean
lines, so the timed kernel pays no write-back of the flush).  `value` = GTEPS = directed nnz per
second / 1e9 with all inputs resident in HBM; `e2e` repeats the step through
the public API with x copied from pinned host memory and y read back inside
the timed region.

--impl reference times the reference's CPU stand-in on the host cores: the
reference has no CPU SpMV, so its arm is the oracle's FP32 CSR SpMV (OpenMP
over rows), on a bounded row sample of the same graph.
"""
from __future__ import annotations

import argparse
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
    p = ROOT / "profiles" / f"merge_spmv_full_full_rmat20_T{T}.md"
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


def time_spmv(torch, A, x, y, steps, warmup, flush, stream):
    for _ in range(warmup):
        A.spmv_bin_full_full(x, y)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    launches = 0
    lib = A._lib if hasattr(A, "_lib") else None
    for k in range(steps):
        flush_l2(flush)
        evs[k][0].record(stream)
        A.spmv_bin_full_full(x, y)
        evs[k][1].record(stream)
        launches += lib.b2sr_last_launch_count() if lib else 0
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in evs]
    return ms, launches


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
    rng = np.random.default_rng(X_SEED)
    x_np = rng.random(g.ncols, dtype=np.float32)
    x = torch.from_numpy(x_np).to(dev)
    flush = torch.ones(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    # tile-size sweep (part of the autotuning; every size reported)
    tiles = [int(t) for t in args.tiles.split(",")]
    sweep = {}
    mats = {}
    for T in tiles:
        t0 = time.time()
        A = pkg.B2SRMatrix.from_graph(g, T, device=dev)
        torch.cuda.synchronize()
        pack_s = time.time() - t0
        A._lib = lib
        y = torch.empty(A.padded_rows(), device=dev)
        ms, _ = time_spmv(torch, A, x, y, steps=20, warmup=5, flush=flush, stream=stream)
        sweep[T] = {"ms": statistics.median(ms), "nblocks": A.nblocks, "pack_s": round(pack_s, 3),
                    "algo_bytes": algorithmic_bytes(A, T)}
        mats[T] = A
    T = min(sweep, key=lambda t: sweep[t]["ms"]) if args.tile == 0 else args.tile
    A = mats[T]
    for t, m in mats.items():
        if t != T:
            m.close()
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
        ms, launches = time_spmv(torch, A, x, y, args.steps, args.warmup, flush, stream)
        t_wall = time.time() - t_wall
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = clk.summary()
    ms_step = sum(ms) / len(ms)
    if world > 1:
        t = torch.tensor([ms_step], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_step = float(t.item())
    nnz = g.nnz
    gteps = nnz / (ms_step * 1e-3) / 1e9 * world

    # e2e: public API with host buffers, copies inside the timed region
    x_host = torch.from_numpy(x_np).pin_memory()
    y_host = torch.empty(A.padded_rows(), dtype=torch.float32).pin_memory()
    xd = torch.empty_like(x)
    for _ in range(max(args.warmup, 3)):
        xd.copy_(x_host, non_blocking=True)
        A.spmv_bin_full_full(xd, y)
        y_host.copy_(y, non_blocking=True)
    torch.cuda.synchronize()
    e2e_steps = min(args.steps, 500)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        xd.copy_(x_host, non_blocking=True)
        A.spmv_bin_full_full(xd, y)
        y_host.copy_(y, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / e2e_steps
    e2e = {"value": round(nnz / (e2e_ms * 1e-3) / 1e9 * world, 3), "unit": "GTEPS",
           "ms_per_step": round(e2e_ms, 5), "h2d_bytes_per_step": int(x_host.numel() * 4),
           "d2h_bytes_per_step": int(y_host.numel() * 4), "steps": e2e_steps,
           "note": "L2 not flushed; x H2D + SpMV + y D2H per step"}

    # cuSPARSE CSR SpMV (the reference's own baseline) on the same graph and GPU
    cus = None
    try:
        crow = torch.from_numpy(g.rowptr).to(dev)
        col = torch.from_numpy(g.colind).to(dev)
        vals = torch.ones(g.nnz, device=dev)
        Acsr = torch.sparse_csr_tensor(crow, col, vals, size=(g.nrows, g.ncols))
        yc = torch.mv(Acsr, x)
        for _ in range(5):
            torch.mv(Acsr, x)
        torch.cuda.synchronize()
        cms = []
        for _ in range(50):
            flush_l2(flush)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            torch.mv(Acsr, x)
            b.record(stream)
            cms.append((a, b))
        torch.cuda.synchronize()
        cm = statistics.median(a.elapsed_time(b) for a, b in cms)
        same = float((yc - y[: g.nrows]).abs().max() / yc.abs().max())
        cus = {"ms": round(cm, 5), "gteps": round(nnz / (cm * 1e-3) / 1e9, 3),
               "bytes": 4 * (g.nrows + 1) + 8 * nnz + 4 * g.ncols + 4 * g.nrows,
               "max_rel_diff_vs_b2sr": same, "api": "torch.mv(sparse_csr) -> cusparseSpMV"}
        del Acsr, vals
    except Exception as e:  # pragma: no cover - reported, not fatal
        cus = {"error": repr(e)[:200]}

    peak, peak_kind = load_peaks()
    algo = algorithmic_bytes(A, T)
    achieved = algo / (ms_step * 1e-3) / 1e9
    traffic = traffic_from_profile(T)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s",
                "algorithmic_bytes_per_launch": algo,
                "timed": "one b2sr_spmv_bin_full_full call per step (CUDA events)"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(g, x_np, budget_s=args.cpu_seconds)

    line = {
        "metric": "B2SR SpMV GTEPS (bin_full_full, single vector)",
        "value": round(gteps, 3), "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 5), "higher_is_better": True,
        "scaling": "weak" if world > 1 else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded R-MAT)",
        "config": {"workload": f"rmat_s20_ef16_bin_full_full_T{T}", "graph": "R-MAT",
                   "scale": RMAT["scale"], "edge_factor": RMAT["edge_factor"],
                   "abc": [RMAT["a"], RMAT["b"], RMAT["c"]], "nrows": g.nrows, "nnz": nnz,
                   "tile_dim": T, "nblocks": A.nblocks, "variant": "bin_full_full",
                   "l2": "flushed between steps (256 MB read, outside the timed events)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "tile_sweep": {str(k): v for k, v in sweep.items()},
                   "launch": dict(zip(("threads", "items_per_thread", "ctas_per_sm"),
                                      A.get_launch("bin_full_full"))),
                   "graph_gen_s": round(gen_s, 2)},
        "roofline": roofline,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "baselines": {"cusparse_csr_spmv_fp32": cus},
        "wall_s_timed_loop": round(t_wall, 3),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
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
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import __graft_entry__ as entry

    pkg = entry.load_package()
    g, _ = make_graph(pkg)
    x_np = np.random.default_rng(X_SEED).random(g.ncols, dtype=np.float32)
    orc = entry.load_oracle()
    # bound the sample so that W + K steps stay within ~2 minutes
    y = np.zeros(g.nrows, np.float32)
    t0 = time.perf_counter()
    _, used = orc.csr_spmv_f32_omp(g.rowptr, g.colind, g.nrows, x_np, y)
    t_full = time.perf_counter() - t0
    budget = 120.0
    frac = min(1.0, budget / max(t_full * (args.steps + args.warmup), 1e-9))
    nrows = max(1, int(g.nrows * frac))
    rp_s = g.rowptr[: nrows + 1]
    ys = np.zeros(nrows, np.float32)
    for _ in range(args.warmup):
        orc.csr_spmv_f32_omp(rp_s, g.colind, nrows, x_np, ys)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        orc.csr_spmv_f32_omp(rp_s, g.colind, nrows, x_np, ys)
        times.append(time.perf_counter() - t0)
    per = sum(times) / len(times)
    nnz = int(rp_s[-1])
    val = nnz / per / 1e9
    line = {
        "impl": "reference",
        "metric": "B2SR SpMV GTEPS (bin_full_full, single vector)",
        "value": round(val, 4), "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(per * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded R-MAT)",
        "config": {"workload": "rmat_s20_ef16_bin_full_full (CSR on host cores)", "nrows": g.nrows,
                   "nnz": g.nnz},
        "cpu_baseline": {"value": round(val, 4), "unit": "GTEPS", "cores": int(used), "kind": "port",
                         "sample": f"rows [0, {nrows}) of {g.nrows} ({nnz} nnz) per step; the reference "
                                   f"has no CPU SpMV, so this is the oracle's FP32 CSR SpMV (OpenMP)"},
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
    ap.add_argument("--tiles", default="4,8,16,32")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
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
