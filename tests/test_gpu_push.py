"""Direction-optimised bit-vector products: the push form (through the cached
transpose) and the device-side auto choice give the pull kernels' results bit
for bit, across the graph zoo, every tile size, sparse and dense frontiers,
accumulate, the masked BFS step and CUDA-graph capture."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from gpu_util import from_np_words, graph_zoo, to_np_words

pytestmark = pytest.mark.gpu

DIRECTIONS = ("pull", "push", "auto")
BIT_VARIANTS = ("bin_bin_bin", "bin_bin_count", "bin_bin_full")


@pytest.fixture(scope="module")
def zoo(pkg):
    return graph_zoo(pkg)


def _frontier(orc, A, density, seed):
    nbc = A.nblockcols
    T = A.tile_dim
    xbool = np.zeros(nbc * T, np.float32)
    xbool[: A.ncols] = np.random.default_rng(seed).random(A.ncols) < density
    return orc.pack_vec_bits(xbool, T)


def _set_direction(A, direction):
    for v in BIT_VARIANTS:
        A.set_launch(v, direction=direction)


def _products(A, xbt, mask_t):
    T = A.tile_dim
    return {
        "bits": to_np_words(A.spmv_bin_bin_bin(xbt), T),
        "masked": to_np_words(A.spmv_bin_bin_bin_masked(xbt, mask_t), T),
        "count": A.spmv_bin_bin_count(xbt).cpu().numpy(),
        "full": A.spmv_bin_bin_full(xbt).cpu().numpy(),
    }


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_push_and_auto_equal_pull_and_oracle(pkg, orc, cuda, zoo, T):
    for name, g in zoo.items():
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
        mask = orc.pack_vec_bits((np.random.default_rng(7).random(A.padded_rows()) < 0.3).astype(np.float32), T)
        mask_t = from_np_words(mask, T, cuda)
        for density in (0.0, 0.002, 0.02, 0.5):
            xb = _frontier(orc, A, density, seed=int(density * 1000) + T)
            xbt = from_np_words(xb, T, cuda)
            want = {
                "bits": orc.bmv_bin_bin_bin(T, brp, bci, tiles, xb),
                "masked": orc.bmv_bin_bin_bin_masked(T, brp, bci, tiles, xb, mask),
                "count": orc.bmv_bin_bin_count(T, brp, bci, tiles, xb),
                "full": orc.bmv_bin_bin_full(T, brp, bci, tiles, xb),
            }
            for direction in DIRECTIONS:
                _set_direction(A, direction)
                got = _products(A, xbt, mask_t)
                for k in want:
                    np.testing.assert_array_equal(got[k], want[k],
                                                  err_msg=f"{name} T={T} d={density} {direction} {k}")
        A.close()


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_push_accumulate(pkg, orc, cuda, zoo, T):
    g = zoo["rmat_s12"]
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
    xb = _frontier(orc, A, 0.01, seed=3)
    xbt = from_np_words(xb, T, cuda)
    b0 = orc.pack_vec_bits((np.random.default_rng(2).random(A.padded_rows()) < 0.2).astype(np.float32), T)
    c0 = np.arange(A.padded_rows(), dtype=np.int32)
    f0 = np.random.default_rng(4).random(A.padded_rows(), dtype=np.float32)
    for direction in ("push", "auto"):
        _set_direction(A, direction)
        b = from_np_words(b0.copy(), T, cuda)
        A.spmv_bin_bin_bin(xbt, b, accumulate=True)
        np.testing.assert_array_equal(to_np_words(b, T), orc.bmv_bin_bin_bin(T, brp, bci, tiles, xb, b0, True))
        c = torch.from_numpy(c0.copy()).to(cuda)
        A.spmv_bin_bin_count(xbt, c, accumulate=True)
        np.testing.assert_array_equal(c.cpu().numpy(), orc.bmv_bin_bin_count(T, brp, bci, tiles, xb, c0, True))
        # FP32 counts with accumulate take the pull (one rounding per entry)
        f = torch.from_numpy(f0.copy()).to(cuda)
        A.spmv_bin_bin_full(xbt, f, accumulate=True)
        _set_direction(A, "pull")
        f_pull = torch.from_numpy(f0.copy()).to(cuda)
        A.spmv_bin_bin_full(xbt, f_pull, accumulate=True)
        np.testing.assert_array_equal(f.cpu().numpy(), f_pull.cpu().numpy())
    A.close()


def test_push_on_larger_graph_matches_pull(pkg, cuda):
    """R-MAT scale 16: push and auto equal pull at frontier densities around
    the switch point, and the bit product equals the count product's support."""
    g = pkg.rmat(16, 16, seed=9)
    for T in (4, 8, 32):
        A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
        for density in (0.0005, 0.005, 0.05, 0.3):
            xbool = (torch.rand(A.nblockcols * T, generator=torch.Generator().manual_seed(T), device="cpu")
                     < density).float()
            xbool[A.ncols:] = 0
            xbt = pkg.pack_vec_bits(xbool.to(cuda), T)
            res = {}
            for direction in DIRECTIONS:
                _set_direction(A, direction)
                res[direction] = (A.spmv_bin_bin_bin(xbt).clone(), A.spmv_bin_bin_count(xbt).clone())
            for direction in ("push", "auto"):
                assert torch.equal(res[direction][0], res["pull"][0]), (T, density, direction)
                assert torch.equal(res[direction][1], res["pull"][1]), (T, density, direction)
            support = pkg.unpack_vec_bits(res["pull"][0], T, A.padded_rows()) != 0
            assert torch.equal(support, res["pull"][1] != 0), (T, density)
        A.close()


def test_bfs_levels_agree_across_directions(pkg, cuda):
    """A masked BFS (next = A.frontier AND NOT visited) reaches the same levels
    with pull, push and auto; the frontier passes from sparse to dense and back."""
    g = pkg.rmat(14, 8, seed=12)
    T = 8
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    n = A.padded_rows()
    levels = {}
    for direction in DIRECTIONS:
        _set_direction(A, direction)
        f = torch.zeros(n, device=cuda)
        f[0] = 1
        fb = pkg.pack_vec_bits(f, T)
        visited = fb.clone()
        lev = torch.full((n,), -1, dtype=torch.int32, device=cuda)
        lev[0] = 0
        for depth in range(1, 64):
            nxt = A.spmv_bin_bin_bin_masked(fb, visited)
            newly = pkg.unpack_vec_bits(nxt, T, n) != 0
            if not bool(newly.any()):
                break
            lev[newly] = depth
            visited = visited | nxt
            fb = nxt
        levels[direction] = lev.cpu()
    assert torch.equal(levels["push"], levels["pull"])
    assert torch.equal(levels["auto"], levels["pull"])
    assert int((levels["pull"] >= 0).sum()) > 1
    A.close()


def test_auto_direction_under_graph_capture(pkg, orc, cuda, zoo):
    """Auto keeps working inside a captured graph: before the transpose exists
    it pulls; once built (outside the capture), the replayed graph chooses per
    replay from the x in its buffer."""
    g = zoo["rmat_s12"]
    T = 4
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
    _set_direction(A, "auto")
    xb_sparse = _frontier(orc, A, 0.002, seed=1)
    xb_dense = _frontier(orc, A, 0.5, seed=2)
    x = from_np_words(xb_sparse, T, cuda)
    y = torch.zeros(A.nblockrows, dtype=x.dtype, device=cuda)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    _set_direction(A, "pull")
    with torch.cuda.stream(s):
        A.spmv_bin_bin_bin(x, y)  # plans and scratch for this stream, no transpose yet
    torch.cuda.current_stream().wait_stream(s)
    _set_direction(A, "auto")
    gr = torch.cuda.CUDAGraph()
    with torch.cuda.graph(gr, stream=s):
        A.spmv_bin_bin_bin(x, y)
    gr.replay()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(to_np_words(y, T), orc.bmv_bin_bin_bin(T, brp, bci, tiles, xb_sparse))
    A.transpose()  # built outside any capture
    with torch.cuda.stream(s):
        A.spmv_bin_bin_bin(x, y)  # scratch for the push on this stream
    torch.cuda.current_stream().wait_stream(s)
    gr2 = torch.cuda.CUDAGraph()
    with torch.cuda.graph(gr2, stream=s):
        A.spmv_bin_bin_bin(x, y)
    for xb in (xb_sparse, xb_dense, xb_sparse):
        x.copy_(from_np_words(xb, T, cuda))
        y.fill_(0x5)
        gr2.replay()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(to_np_words(y, T), orc.bmv_bin_bin_bin(T, brp, bci, tiles, xb))
    A.close()


def test_forced_push_without_transpose_in_capture_is_refused(pkg, cuda, zoo):
    g = zoo["er_4096_d16"]
    A = pkg.B2SRMatrix.from_graph(g, 8, device=cuda)
    A.set_launch("bin_bin_bin", direction="push")
    x = torch.zeros(A.nblockcols, dtype=torch.uint8, device=cuda)
    y = torch.zeros(A.nblockrows, dtype=torch.uint8, device=cuda)
    s = torch.cuda.Stream()
    gr = torch.cuda.CUDAGraph()
    refused = False
    with torch.cuda.graph(gr, stream=s):
        try:
            A.spmv_bin_bin_bin(x, y)
        except pkg.B2SRError as e:
            refused = e.status == 5  # B2SR_ERR_NOT_SUPPORTED
        torch.zeros(1, device=cuda).add_(1)  # keep the captured graph non-empty
    assert refused
    A.close()


def test_direction_round_trips_and_rejects_bad_values(pkg, cuda, zoo):
    A = pkg.B2SRMatrix.from_graph(zoo["ragged_1001"], 4, device=cuda)
    for direction in DIRECTIONS:
        A.set_launch("bin_bin_count", direction=direction)
        assert A.get_launch("bin_bin_count")[6] == direction
    with pytest.raises(KeyError):
        A.set_launch("bin_bin_count", direction="sideways")
    A.close()


def test_push_on_matrix_without_tiles_accepts_null_x(pkg, cuda, zoo):
    """A matrix with no tiles never reads x, in either direction: NULL x is
    accepted and y comes back zero."""
    import ctypes as C
    lib = pkg._lib.load()
    A = pkg.B2SRMatrix.from_graph(zoo["empty_rows_only"], 8, device=cuda)
    assert A.nblocks == 0
    for direction in DIRECTIONS:
        A.set_launch("bin_bin_bin", direction=direction)
        y = torch.full((A.nblockrows,), 0xFF, dtype=torch.uint8, device=cuda)
        rc = lib.b2sr_spmv_bin_bin_bin(A.handle, None, C.c_void_p(y.data_ptr()), 0,
                                       C.c_void_p(torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        assert rc == 0, direction
        assert int(y.sum()) == 0, direction
    A.close()


@pytest.mark.parametrize("T", [4, 8, 16, 32])
def test_auto_direction_hint_sequences(pkg, orc, cuda, zoo, T):
    """Outside a capture the auto direction starts from the device's last
    decision for the same kind (a hint): a dense frontier after a dense one
    runs the pull at once (the next decision counted beside it), a sparse one
    after a sparse one the push, and a switch costs a device-side launch.
    Every step of sequences that cross the threshold both ways equals the
    oracle, for all four bit kinds."""
    g = zoo["rmat_s12"]
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
    mask = orc.pack_vec_bits((np.random.default_rng(5).random(A.padded_rows()) < 0.3).astype(np.float32), T)
    mask_t = from_np_words(mask, T, cuda)
    _set_direction(A, "auto")
    for step, density in enumerate((0.5, 0.5, 0.5, 0.002, 0.002, 0.5, 0.002, 0.6, 0.6, 0.0, 0.5)):
        xb = _frontier(orc, A, density, seed=100 + step)
        xbt = from_np_words(xb, T, cuda)
        want = {
            "bits": orc.bmv_bin_bin_bin(T, brp, bci, tiles, xb),
            "masked": orc.bmv_bin_bin_bin_masked(T, brp, bci, tiles, xb, mask),
            "count": orc.bmv_bin_bin_count(T, brp, bci, tiles, xb),
            "full": orc.bmv_bin_bin_full(T, brp, bci, tiles, xb),
        }
        got = _products(A, xbt, mask_t)
        torch.cuda.synchronize()
        for k in want:
            np.testing.assert_array_equal(got[k], want[k], err_msg=f"T={T} step {step} d={density} {k}")
    A.close()


@pytest.mark.parametrize("T", [4, 16])
def test_auto_device_launched_pull_is_stream_ordered(pkg, orc, cuda, zoo, T):
    """After a sparse frontier (push hint) a dense one makes the push kernel's
    gate launch the pull from the device: work issued next on the same stream
    (a copy of y) must see the pull's result, with no device-wide sync in
    between."""
    g = zoo["rmat_s12"]
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    A.transpose()
    brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
    xs = from_np_words(_frontier(orc, A, 0.002, seed=11), T, cuda)
    xb_dense = _frontier(orc, A, 0.5, seed=12)
    xd = from_np_words(xb_dense, T, cuda)
    want = orc.bmv_bin_bin_bin(T, brp, bci, tiles, xb_dense)
    _set_direction(A, "auto")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    x = torch.empty_like(xs)
    y = torch.empty(A.nblockrows, dtype=xs.dtype, device=cuda)
    y2 = torch.empty_like(y)
    for _ in range(3):
        with torch.cuda.stream(s):
            x.copy_(xs)
            A.spmv_bin_bin_bin(x, y)
            x.copy_(xd)
            y.zero_()
            A.spmv_bin_bin_bin(x, y)
            y2.copy_(y)
        s.synchronize()
        np.testing.assert_array_equal(to_np_words(y2, T), want)
    A.close()


def test_auto_direction_two_host_threads(pkg, orc, cuda, zoo):
    """Two host threads run auto-direction products of one matrix on their own
    streams with alternating sparse and dense frontiers: they share the
    matrix's hint and get their own side streams, counters and scratch, and
    every result equals the oracle."""
    import threading

    g = zoo["rmat_s12"]
    T = 4
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    A.transpose()
    brp, bci, tiles = orc.csr_to_b2sr(g.rowptr, g.colind, g.nrows, T)
    _set_direction(A, "auto")
    frontiers = [_frontier(orc, A, d, seed=200 + i) for i, d in enumerate((0.002, 0.5, 0.002, 0.6, 0.0, 0.5))]
    wants = [orc.bmv_bin_bin_bin(T, brp, bci, tiles, xb) for xb in frontiers]
    xs = [from_np_words(xb, T, cuda) for xb in frontiers]
    torch.cuda.synchronize()
    errors = []

    def worker(offset):
        try:
            s = torch.cuda.Stream()
            for rep in range(4):
                for i in range(len(xs)):
                    k = (i + offset) % len(xs)
                    with torch.cuda.stream(s):
                        y = torch.empty(A.nblockrows, dtype=xs[k].dtype, device=cuda)
                        A.spmv_bin_bin_bin(xs[k], y)
                    s.synchronize()
                    if not np.array_equal(to_np_words(y, T), wants[k]):
                        errors.append((offset, rep, k))
        except Exception as e:  # reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(o,)) for o in (0, 3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors[:5]
    A.close()
