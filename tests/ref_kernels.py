"""Launcher of the reference's own CUDA kernels (test infrastructure).

oracle/_ref/bsrbmv_ref.cubin is the reference's bmv_eval/backend/bsrbmv.cu,
unmodified, compiled for sm_103a by oracle/build_oracle.py; kernels.txt lists
its mangled kernel names.  Kernels are launched through the CUDA driver API
with the grid/block shapes of the reference drivers
(bmv_eval/test_bin_bin_bin.cu:325-369, test_bin_bin_full.cu:311-346,
test_bin_full_full.cu:274-296, csr2bsr_batch_bsrbmv.cu:107,230,353,476).

Input conditions under which these kernels are well defined (read from the
source): the bin_bin_* kernels vote with a full-mask ballot inside
`if (row < nblockrows)`, so nblockrows must be a multiple of the tile-rows per
warp (8 for T=4, 4 for T=8, 2 for T=16); the bin_full_full kernels call
__syncthreads() inside per-warp loops, so every tile-row must hold the same
number of tiles and nblockrows must be a multiple of 32; their tail loads read
up to 31 colind entries past a row, so colind is zero-padded.  `check_*`
helpers enforce these before any launch.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parents[1]
CUBIN = ROOT / "oracle" / "_ref" / "bsrbmv_ref.cubin"
NAMES = ROOT / "oracle" / "_ref" / "kernels.txt"


def available() -> bool:
    return CUBIN.exists() and NAMES.exists()


class RefKernels:
    def __init__(self):
        if not available():
            raise RuntimeError("reference cubin not built (oracle/build_oracle.py build_ref)")
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # primary context current on this thread
        self.cu = C.CDLL("libcuda.so.1")
        self.mod = C.c_void_p()
        rc = self.cu.cuModuleLoad(C.byref(self.mod), str(CUBIN).encode())
        if rc != 0:
            raise RuntimeError(f"cuModuleLoad failed: {rc}")
        self.names = {}
        for mangled in NAMES.read_text().split():
            # _Z<len><name>... -> name
            i = 2
            j = i
            while mangled[j].isdigit():
                j += 1
            ln = int(mangled[i:j])
            self.names[mangled[j:j + ln]] = mangled
        self.fns = {}

    def fn(self, name):
        if name not in self.fns:
            f = C.c_void_p()
            rc = self.cu.cuModuleGetFunction(C.byref(f), self.mod, self.names[name].encode())
            if rc != 0:
                raise RuntimeError(f"cuModuleGetFunction({name}) failed: {rc}")
            self.fns[name] = f
        return self.fns[name]

    def launch(self, name, grid, block, args):
        """args: list of (ctypes value) in kernel parameter order."""
        holders = [a if isinstance(a, C._SimpleCData) else C.c_void_p(a) for a in args]
        arr = (C.c_void_p * len(holders))(*[C.cast(C.pointer(h), C.c_void_p) for h in holders])
        gx, gy, gz = grid
        stream = torch.cuda.current_stream().cuda_stream
        rc = self.cu.cuLaunchKernel(self.fn(name), gx, gy, gz, block, 1, 1, 0, C.c_void_p(stream), arr, None)
        if rc != 0:
            raise RuntimeError(f"cuLaunchKernel({name}) failed: {rc}")

    # ---- launch shapes of the reference drivers ------------------------------------
    @staticmethod
    def cubic(x):
        g = int(math.ceil(round(x ** (1.0 / 3.0), 12)))
        while g ** 3 < x:
            g += 1
        return max(g, 1)

    def bmv(self, variant, T, tiles, x, y, rowptr, colind, nb):
        if variant == "bin_full_full":
            g, threads = self.cubic(nb / 32), 1024
        elif variant == "bin_bin_bin":
            g, threads = {4: (self.cubic(nb / 8), 32), 8: (self.cubic(nb / 4), 32),
                          16: (self.cubic(nb / 2), 32), 32: (self.cubic(nb / 32), 1024)}[T]
        elif variant == "bin_bin_full":
            g, threads = {4: (self.cubic(nb / 8), 32), 8: (self.cubic(nb / 4), 32),
                          16: (self.cubic(nb / 2), 32), 32: (self.cubic(nb), 32)}[T]
        else:
            raise ValueError(variant)
        self.launch(f"bmv{T}_{variant}", (g, g, g), threads,
                    [tiles.data_ptr(), x.data_ptr(), y.data_ptr(), rowptr.data_ptr(), colind.data_ptr(),
                     C.c_int(nb)])

    def to_bit_row(self, T, x, out, nb):
        g = {4: self.cubic(nb / 4), 8: self.cubic(nb / 4), 16: self.cubic(nb / 2), 32: self.cubic(nb)}[T]
        self.launch(f"ToBit{T}Row", (g, g, g), 32, [x.data_ptr(), out.data_ptr(), C.c_int(nb)])

    def to_bit_col(self, T, dense_tiles, out, nt):
        if T == 32:
            self.launch("ToBit32Col", (1, nt, 1), 32,
                        [dense_tiles.data_ptr(), out.data_ptr(), C.c_int(32), C.c_int(nt * 32)])
        else:
            per = {4: 64, 8: 16, 16: 4}[T]
            self.launch(f"ToBit{T}Col", (1, (nt + per - 1) // per, 1), 32,
                        [dense_tiles.data_ptr(), out.data_ptr(), C.c_int(nt)])


# ---- buffer sizing that keeps every reference access in bounds -------------------------
def x_float_len(nb, T):
    """Floats ToBit{T}Row may read: ceil(nb/4)*32 for T <= 8, ceil(nb/2)*32, nb*32."""
    return {4: -(-nb // 4) * 16, 8: -(-nb // 4) * 32, 16: -(-nb // 2) * 32, 32: nb * 32}[T] + 64


def xbits_len(nb, T):
    return {4: -(-nb // 4) * 4, 8: -(-nb // 4) * 4, 16: -(-nb // 2) * 2, 32: nb}[T] + 64


def packed_tiles_len(nt, T):
    """Words ToBit{T}Col writes (it fills whole groups of 64 / 16 / 4 / 1 tiles)."""
    per = {4: 64, 8: 16, 16: 4, 32: 1}[T]
    return -(-nt // per) * per * T + 64


def check_bits_input(T, nb):
    per_warp = {4: 8, 8: 4, 16: 2, 32: 1}[T]
    assert nb % per_warp == 0, "nblockrows must fill whole warps for the reference bin_bin kernels"


def check_full_full_input(rowptr: np.ndarray):
    nb = len(rowptr) - 1
    loads = np.diff(rowptr)
    assert nb % 32 == 0, "nblockrows must be a multiple of 32 for the reference bin_full_full kernels"
    assert loads.size == 0 or np.all(loads == loads[0]), "uniform tiles per tile-row needed"


def dense_tiles(T, bcolind_rows, tiles_words):
    """Expand packed tiles (our layout) to row-major float tiles, as cusparseScsr2bsr emits them."""
    nt = len(tiles_words) // T
    w = tiles_words.astype(np.uint64).reshape(nt, T)
    cols = np.arange(T, dtype=np.uint64)
    bits = (w[:, :, None] >> (np.uint64(T - 1) - cols)[None, None, :]) & np.uint64(1)
    return bits.astype(np.float32).reshape(-1)
