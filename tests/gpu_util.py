"""Helpers shared by the GPU tests: graphs, oracle comparisons, tolerances."""
from __future__ import annotations

import numpy as np
import torch

# bin_full_full accuracy bar: |y - y64| <= REL_TOL * sum_j |A_ij x_j| per row,
# against the FP64 CSR oracle (a 1e-5 relative bound for FP32 results, taken
# against the row's absolute-value sum so rows whose terms cancel keep a fair scale).
REL_TOL = 1e-5


def to_np_words(t: torch.Tensor, T: int) -> np.ndarray:
    a = t.detach().cpu().numpy()
    return a.view({4: np.uint8, 8: np.uint8, 16: np.uint16, 32: np.uint32}[T])


def from_np_words(a: np.ndarray, T: int, device) -> torch.Tensor:
    dt = {4: np.uint8, 8: np.uint8, 16: np.int16, 32: np.int32}[T]
    return torch.from_numpy(np.ascontiguousarray(a).view(dt)).to(device)


def full_full_error(orc, g, x: np.ndarray, y: np.ndarray) -> float:
    """max_i |y_i - y64_i| / max(sum_j |x_j| over row i, tiny)."""
    y64 = orc.csr_spmv_f64(g.rowptr, g.colind, g.nrows, x)
    scale = orc.csr_spmv_abs_f64(g.rowptr, g.colind, g.nrows, x)
    return float((np.abs(y[: g.nrows].astype(np.float64) - y64) / np.maximum(scale, 1e-30)).max(initial=0.0))


def graph_zoo(pkg):
    """Small graphs covering the edge cases of packing and multiplying."""
    zoo = {
        "er_4096_d16": pkg.erdos_renyi(4096, 16.0, seed=1),
        "rmat_s12": pkg.rmat(12, 16, seed=3),
        "ragged_1001": pkg.erdos_renyi(1001, 5.0, seed=4),
        "rect_70x333": pkg.from_edges(np.random.default_rng(5).integers(0, 70, 900),
                                      np.random.default_rng(6).integers(0, 333, 900), nrows=70, ncols=333),
        "single_row": pkg.from_edges([0, 0, 0], [3, 17, 40], nrows=1, ncols=64),
        "empty_rows_only": pkg.from_edges([], [], nrows=37, ncols=37),
    }
    # a hub row spanning many threads, warps and CTAs, among empty rows
    n = 40000
    hub_cols = np.arange(1, n, 2)
    rows = np.concatenate([np.full(hub_cols.size, 5), [39999, 7]])
    cols = np.concatenate([hub_cols, [0, 39998]])
    zoo["hub_40000"] = pkg.from_edges(rows, cols, nrows=n)
    # dense block: every tile full
    d = 96
    r, c = np.meshgrid(np.arange(d), np.arange(d), indexing="ij")
    zoo["dense_96"] = pkg.from_edges(r.ravel(), c.ravel(), nrows=d, drop_self_loops=False)
    return zoo
