"""Generates the golden fixtures in this folder by running the REFERENCE's own
kernels (oracle/_ref/bsrbmv_ref.cubin, built from the reference's
bmv_eval/backend/bsrbmv.cu) on a GPU.

For every tile size T and two seeded cases it records:
  * the reference packer's bit tiles: dense row-major float tiles (what
    cusparseScsr2bsr hands to ToBit{T}Col, csr2bsr_batch_bsrbmv.cu:100-107),
    built here with numpy straight from the CSR, packed by ToBit{T}Col;
  * the reference vector packer's bits: ToBit{T}Row of x (test_bin_bin_bin.cu:249-282);
  * one launch of bmv{T}_bin_bin_bin, bmv{T}_bin_bin_full and (uniform case
    only) bmv{T}_bin_full_full on those buffers, y zero-initialised.
Cases: "rmat" (R-MAT scale 10, irregular rows; nblockrows a multiple of 8) and
"uniform" (every tile-row holds the same number of tiles, nblockrows = 64),
the input conditions under which the reference kernels are well defined (see
tests/ref_kernels.py).

Usage (GPU machine, reference cubin prebuilt):
    python tests/golden/make_golden.py --out tests/golden
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import torch  # noqa: E402

import __graft_entry__ as entry  # noqa: E402
import ref_kernels as rk  # noqa: E402

WORD_NP = {4: np.uint8, 8: np.uint8, 16: np.uint16, 32: np.uint32}
WORD_T = {4: torch.uint8, 8: torch.uint8, 16: torch.int16, 32: torch.int32}


def b2sr_structure_numpy(rowptr, colind, nrows, T):
    """Tile list of a CSR in cusparseScsr2bsr order (ascending tile-column per tile-row)."""
    nb = (nrows + T - 1) // T
    rows = np.repeat(np.arange(nrows), np.diff(rowptr))
    key = (rows // T).astype(np.int64) * (1 << 32) + colind // T
    uk = np.unique(key)
    btr, btc = (uk >> 32).astype(np.int64), (uk & 0xFFFFFFFF).astype(np.int64)
    brp = np.searchsorted(btr, np.arange(nb + 1)).astype(np.int32)
    dense = np.zeros((uk.size, T, T), np.float32)
    tix = np.searchsorted(uk, key)
    dense[tix, rows % T, colind % T] = 1.0
    return brp, btc.astype(np.int32), dense.reshape(-1)


def uniform_case(T, nb=64, per_row=7, seed=0):
    rng = np.random.default_rng(seed + T)
    rows, cols = [], []
    for tr in range(nb):
        tcs = np.sort(rng.choice(nb, size=per_row, replace=False))
        for tc in tcs:
            bits = rng.random((T, T)) < 0.25
            bits[rng.integers(T), rng.integers(T)] = True
            r, c = np.nonzero(bits)
            rows.extend((tr * T + r).tolist())
            cols.extend((tc * T + c).tolist())
    n = nb * T
    pkg = entry.load_package()
    return pkg.from_edges(rows, cols, nrows=n, ncols=n, drop_self_loops=False)


def run_case(ref, g, T, name, seed, full_full):
    dev = torch.device("cuda")
    nb = (g.nrows + T - 1) // T
    rk.check_bits_input(T, nb)
    brp, bci, dense = b2sr_structure_numpy(g.rowptr, g.colind, g.nrows, T)
    nt = len(bci)
    if full_full:
        rk.check_full_full_input(brp)
    rng = np.random.default_rng(seed)
    x = np.zeros(rk.x_float_len(nb, T), np.float32)
    x[: g.ncols] = rng.random(g.ncols, dtype=np.float32)
    xbool = np.zeros_like(x)
    xbool[: g.ncols] = (rng.random(g.ncols) < 0.5).astype(np.float32)

    d_dense = torch.from_numpy(dense).to(dev)
    d_tiles = torch.zeros(rk.packed_tiles_len(nt, T), dtype=WORD_T[T], device=dev)
    ref.to_bit_col(T, d_dense, d_tiles, nt)
    d_xb = torch.zeros(rk.xbits_len(nb, T), dtype=WORD_T[T], device=dev)
    ref.to_bit_row(T, torch.from_numpy(xbool).to(dev), d_xb, nb)
    d_rp = torch.from_numpy(brp).to(dev)
    d_ci = torch.zeros(nt + 64, dtype=torch.int32, device=dev)  # zero padding past the last tile
    d_ci[:nt] = torch.from_numpy(bci).to(dev)
    y_bbb = torch.zeros(nb + 64, dtype=WORD_T[T], device=dev)
    ref.bmv("bin_bin_bin", T, d_tiles, d_xb, y_bbb, d_rp, d_ci, nb)
    y_bbf = torch.zeros(nb * T + 64, dtype=torch.float32, device=dev)
    ref.bmv("bin_bin_full", T, d_tiles, d_xb, y_bbf, d_rp, d_ci, nb)
    out = {}
    if full_full:
        y_bff = torch.zeros(nb * T + 64, dtype=torch.float32, device=dev)
        ref.bmv("bin_full_full", T, d_tiles, torch.from_numpy(x).to(dev), y_bff, d_rp, d_ci, nb)
        out["ref_y_bff"] = y_bff[: nb * T].cpu().numpy()
    torch.cuda.synchronize()
    nbc = (g.ncols + T - 1) // T
    out.update({
        "T": np.int32(T), "nrows": np.int32(g.nrows), "ncols": np.int32(g.ncols),
        "csr_rowptr": g.rowptr, "csr_colind": g.colind,
        "b2sr_rowptr": brp, "b2sr_colind": bci,
        "x": x[: g.ncols], "xbool": xbool[: g.ncols],
        "ref_tiles": d_tiles[: nt * T].cpu().numpy().view(WORD_NP[T]),
        "ref_xbits": d_xb[:nbc].cpu().numpy().view(WORD_NP[T]),
        "ref_y_bbb": y_bbb[:nb].cpu().numpy().view(WORD_NP[T]),
        "ref_y_bbf": y_bbf[: nb * T].cpu().numpy(),
    })
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(HERE))
    args = ap.parse_args()
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    entry.build()
    pkg = entry.load_package()
    ref = rk.RefKernels()
    for T in (4, 8, 16, 32):
        g = pkg.rmat(10, 8, seed=100 + T)
        np.savez_compressed(out / f"ref_rmat10_T{T}.npz", **run_case(ref, g, T, "rmat", 200 + T, False))
        gu = uniform_case(T)
        np.savez_compressed(out / f"ref_uniform_T{T}.npz", **run_case(ref, gu, T, "uniform", 300 + T, True))
        print("T", T, "done", flush=True)


if __name__ == "__main__":
    main()
