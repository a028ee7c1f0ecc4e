// Merge-path B2SR multiply, shared by all variants.
//
// Work decomposition (merge-based SpMV, Merrill & Garland, SC'16, restated for
// B2SR): the work list is the merge of the nb tile-row ends with the nt tiles,
// nb + nt items.  A persistent grid splits it into equal shares (the start
// coordinate of every CTA is computed once per matrix by the partition
// kernel).  A CTA walks its share in sub-chunks of THREADS*ITEMS items; every
// thread takes ITEMS consecutive items, so each thread reads a contiguous run
// of tiles.  Consuming a tile adds its contribution to the thread's T row
// accumulators; consuming a row end writes the tile-row's T outputs.
//
// A tile-row that spans several threads leaves partial sums ("carries").  They
// are combined by a segmented scan over the block in thread order, so every
// output is the sum of its tiles in one fixed order: the result is bitwise
// reproducible and there are no float atomics (the reference's T < 32
// bin_full_full kernels use atomicAdd, bsrbmv.cu:895,971,1036).  The carry of
// the last open tile-row moves to the next sub-chunk inside the CTA, and the
// CTA's final carry goes to a scratch array that the fix-up kernel adds in CTA
// order.
#pragma once

#include "b2sr_common.cuh"

namespace b2sr {

// ---- tile loads -------------------------------------------------------------------
// The T row words of tile j, each widened to 32 bits (row r of the tile in
// rows[r]; bit T-1-c = column c).  Read-only path; a thread's tiles are
// contiguous, so the L1 keeps the line for its next tiles.
template <int T> struct TileRows;

template <> struct TileRows<4> {
    static __device__ __forceinline__ void load(const uint8_t* tiles, long long j, uint32_t (&rows)[4]) {
        const uint32_t w = __ldg(reinterpret_cast<const unsigned int*>(tiles) + j);
#pragma unroll
        for (int r = 0; r < 4; ++r) rows[r] = (w >> (8 * r)) & 0xFu;
    }
};
template <> struct TileRows<8> {
    static __device__ __forceinline__ void load(const uint8_t* tiles, long long j, uint32_t (&rows)[8]) {
        const uint2 w = __ldg(reinterpret_cast<const uint2*>(tiles) + j);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            rows[r] = (w.x >> (8 * r)) & 0xFFu;
            rows[r + 4] = (w.y >> (8 * r)) & 0xFFu;
        }
    }
};
template <> struct TileRows<16> {
    static __device__ __forceinline__ void load(const uint16_t* tiles, long long j, uint32_t (&rows)[16]) {
        const uint4* p = reinterpret_cast<const uint4*>(tiles) + 2 * j;
        const uint4 a = __ldg(p), b = __ldg(p + 1);
        const uint32_t u[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            rows[2 * q] = u[q] & 0xFFFFu;
            rows[2 * q + 1] = u[q] >> 16;
        }
    }
};
template <> struct TileRows<32> {
    static __device__ __forceinline__ void load(const uint32_t* tiles, long long j, uint32_t (&rows)[32]) {
        const uint4* p = reinterpret_cast<const uint4*>(tiles) + 8 * j;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const uint4 a = __ldg(p + q);
            rows[4 * q] = a.x;
            rows[4 * q + 1] = a.y;
            rows[4 * q + 2] = a.z;
            rows[4 * q + 3] = a.w;
        }
    }
};

// ---- vector output helpers -------------------------------------------------------------
template <int T, typename V>
__device__ __forceinline__ void store_row(V* __restrict__ y, int row, const V (&v)[T], int accumulate) {
    V* p = y + (size_t)row * T;
    if (accumulate) {
#pragma unroll
        for (int r = 0; r < T; ++r) p[r] = p[r] + v[r];
    } else {
#pragma unroll
        for (int r = 0; r < T; ++r) p[r] = v[r];
    }
}

// ---- variant ops -----------------------------------------------------------------------
// Each op defines the accumulator of one tile-row (Acc), how a tile updates it,
// how partial accumulators combine, and how a finished tile-row is written
// (emit) or a late carry is added (fix).

// bin_full_full: FP32 x, FP32 y.  Set bits of a tile row are visited in
// ascending column order (as bmv32_bin_full_full does, bsrbmv.cu:1063-1076).
template <int T>
struct OpFullFull {
    using W = typename TileWord<T>::type;
    using X = float;
    using Y = float;
    struct Acc { float v[T]; };
    static __device__ __forceinline__ void zero(Acc& a) {
#pragma unroll
        for (int r = 0; r < T; ++r) a.v[r] = 0.0f;
    }
    static __device__ __forceinline__ void tile(Acc& a, const W* tiles, long long j, int tc,
                                                const X* __restrict__ x) {
        uint32_t rows[T];
        TileRows<T>::load(tiles, j, rows);
        const float* xs = x + (size_t)tc * T;
#pragma unroll
        for (int r = 0; r < T; ++r) {
            uint32_t w = rows[r];
            while (w) {
                const int b = 31 - __clz(w);
                a.v[r] += __ldg(xs + (T - 1 - b));
                w &= ~(1u << b);
            }
        }
    }
    static __device__ __forceinline__ void combine(Acc& a, const Acc& b) {
#pragma unroll
        for (int r = 0; r < T; ++r) a.v[r] += b.v[r];
    }
    static __device__ __forceinline__ void shfl_up(Acc& out, const Acc& a, int o) {
#pragma unroll
        for (int r = 0; r < T; ++r) out.v[r] = __shfl_up_sync(FULL_MASK, a.v[r], o);
    }
    static __device__ __forceinline__ void emit(Y* y, const W*, int row, const Acc& a, int accumulate) {
        store_row<T, float>(y, row, a.v, accumulate);
    }
    static __device__ __forceinline__ void fix(Y* y, const W*, int row, const Acc& a) {
        store_row<T, float>(y, row, a.v, 1);
    }
};

// bin_bin_full / bin_bin_count: bit x, count y (float or int32).  Counts are
// integers, so any order gives the same result.
template <int T, typename YT>
struct OpCount {
    using W = typename TileWord<T>::type;
    using X = W;
    using Y = YT;
    struct Acc { int v[T]; };
    static __device__ __forceinline__ void zero(Acc& a) {
#pragma unroll
        for (int r = 0; r < T; ++r) a.v[r] = 0;
    }
    static __device__ __forceinline__ void tile(Acc& a, const W* tiles, long long j, int tc,
                                                const X* __restrict__ x) {
        uint32_t rows[T];
        TileRows<T>::load(tiles, j, rows);
        const uint32_t xw = __ldg(x + tc);
#pragma unroll
        for (int r = 0; r < T; ++r) a.v[r] += __popc(rows[r] & xw);
    }
    static __device__ __forceinline__ void combine(Acc& a, const Acc& b) {
#pragma unroll
        for (int r = 0; r < T; ++r) a.v[r] += b.v[r];
    }
    static __device__ __forceinline__ void shfl_up(Acc& out, const Acc& a, int o) {
#pragma unroll
        for (int r = 0; r < T; ++r) out.v[r] = __shfl_up_sync(FULL_MASK, a.v[r], o);
    }
    static __device__ __forceinline__ void emit(Y* y, const W*, int row, const Acc& a, int accumulate) {
        Y v[T];
#pragma unroll
        for (int r = 0; r < T; ++r) v[r] = (Y)a.v[r];
        store_row<T, Y>(y, row, v, accumulate);
    }
    static __device__ __forceinline__ void fix(Y* y, const W*, int row, const Acc& a) {
        Y v[T];
#pragma unroll
        for (int r = 0; r < T; ++r) v[r] = (Y)a.v[r];
        store_row<T, Y>(y, row, v, 1);
    }
};

// bin_bin_bin: bit x, bit y; row r of the output word is set when any tile of
// the tile-row has a common bit between its row r and the x word (the
// reference's popc(A & x) > 0 vote, bsrbmv.cu:300-309).  MASKED: y = result
// AND NOT mask, overwriting (bsrbmv.cu:1113-1118).
template <int T, bool MASKED>
struct OpBits {
    using W = typename TileWord<T>::type;
    using X = W;
    using Y = W;
    struct Acc { uint32_t m; };
    static __device__ __forceinline__ void zero(Acc& a) { a.m = 0; }
    static __device__ __forceinline__ void tile(Acc& a, const W* tiles, long long j, int tc,
                                                const X* __restrict__ x) {
        uint32_t rows[T];
        TileRows<T>::load(tiles, j, rows);
        const uint32_t xw = __ldg(x + tc);
#pragma unroll
        for (int r = 0; r < T; ++r) a.m |= ((rows[r] & xw) != 0u ? 1u : 0u) << (T - 1 - r);
    }
    static __device__ __forceinline__ void combine(Acc& a, const Acc& b) { a.m |= b.m; }
    static __device__ __forceinline__ void shfl_up(Acc& out, const Acc& a, int o) {
        out.m = __shfl_up_sync(FULL_MASK, a.m, o);
    }
    static __device__ __forceinline__ void emit(Y* y, const W* mask, int row, const Acc& a, int accumulate) {
        if (MASKED) {
            y[row] = (W)(a.m & ~(uint32_t)mask[row]);
        } else {
            y[row] = (W)(accumulate ? ((uint32_t)y[row] | a.m) : a.m);
        }
    }
    static __device__ __forceinline__ void fix(Y* y, const W* mask, int row, const Acc& a) {
        const uint32_t add = MASKED ? (a.m & ~(uint32_t)mask[row]) : a.m;
        y[row] = (W)((uint32_t)y[row] | add);
    }
};

// Scratch record of one CTA's final carry.
template <class Op>
struct alignas(16) CarryRec {
    int row;
    int pad[3];
    typename Op::Acc val;
};

// ---- partition ---------------------------------------------------------------------------
// starts[c] = merge-path coordinate of diagonal floor(c * (nb + nt) / grid),
// c = 0..grid.  One warp per boundary, 33-ary search: 32 lanes probe 32 evenly
// spaced rows per round, so a 2^20-row search takes 4 rounds of memory latency
// instead of 20.  The predicate "row x has ended before tile d-x-1"
// (rowptr[x+1] <= d-x-1) is true then false along x; the coordinate is the
// first x where it is false.
__global__ void partition_kernel(const int* __restrict__ rowptr, int nb, int grid,
                                 Coord* __restrict__ starts);

// ---- the multiply kernel ----------------------------------------------------------------------
template <class Op, int T, int THREADS, int ITEMS>
struct MergeSmem {
    int rowend[THREADS * ITEMS + 1];
    int wkey[THREADS / 32];
    int wfirst[THREADS / 32];
    typename Op::Acc wacc[THREADS / 32];
    int next_row, next_tile;
    typename Op::Acc carry;
};

template <class Op, int T, int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS)
merge_spmv_kernel(const int* __restrict__ rowptr, const int* __restrict__ colind,
                  const typename Op::W* __restrict__ tiles, int nb,
                  const Coord* __restrict__ starts, const typename Op::X* __restrict__ x,
                  typename Op::Y* __restrict__ y, const typename Op::W* __restrict__ mask,
                  int accumulate, CarryRec<Op>* __restrict__ carries) {
    using Acc = typename Op::Acc;
    constexpr int IPC = THREADS * ITEMS;
    constexpr int NW = THREADS / 32;
    __shared__ MergeSmem<Op, T, THREADS, ITEMS> sm;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nt = rowptr[nb];
    const Coord beg = starts[blockIdx.x];
    const Coord end = starts[blockIdx.x + 1];
    const long long d_end = (long long)end.row + end.tile;
    int i0 = beg.row, j0 = beg.tile;
    Acc carry;
    Op::zero(carry);

    while ((long long)i0 + j0 < d_end) {
        const int n_items = (int)min((long long)IPC, d_end - ((long long)i0 + j0));
        // Row ends of the rows this sub-chunk can reach (at most n_items).
        for (int k = tid; k <= n_items; k += THREADS) {
            const int r = i0 + k;
            sm.rowend[k] = r < nb ? __ldg(rowptr + r + 1) : nt;
        }
        __syncthreads();

        // This thread's start coordinate: merge-path search on the staged row ends.
        const int rd = min(tid * ITEMS, n_items);
        int lo = max(0, rd - (nt - j0)), hi = min(rd, nb - i0);
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (sm.rowend[mid] <= j0 + rd - mid - 1) lo = mid + 1;
            else hi = mid;
        }
        int i = i0 + lo, j = j0 + rd - lo;
        const int my_items = min(ITEMS, n_items - rd);
        Acc acc;
        if (tid == 0) acc = carry;
        else Op::zero(acc);

        for (int k = 0; k < my_items; ++k) {
            if (j < sm.rowend[i - i0]) {
                Op::tile(acc, tiles, j, __ldg(colind + j), x);
                ++j;
            } else {
                Op::emit(y, mask, i, acc, accumulate);
                Op::zero(acc);
                ++i;
            }
        }

        // Segmented inclusive scan of the per-thread carries keyed by the open
        // row; keys are non-decreasing in thread order.
        const int key = i;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int k2 = __shfl_up_sync(FULL_MASK, key, o);
            Acc a2;
            Op::shfl_up(a2, acc, o);
            if (lane >= o && k2 == key) {
                Acc t = a2;
                Op::combine(t, acc);
                acc = t;
            }
        }
        const int first_key = __shfl_sync(FULL_MASK, key, 0);
        if (lane == 31) {
            sm.wkey[warp] = key;
            sm.wfirst[warp] = first_key;
            sm.wacc[warp] = acc;
        }
        __syncthreads();
        if (warp > 0 && key == first_key) {
            Acc pre;
            Op::zero(pre);
            bool any = false;
            for (int w2 = warp - 1; w2 >= 0; --w2) {
                if (sm.wkey[w2] != key) break;
                Acc t = sm.wacc[w2];
                Op::combine(t, pre);
                pre = t;
                any = true;
                if (sm.wfirst[w2] != key) break;
            }
            if (any) {
                Op::combine(pre, acc);
                acc = pre;
            }
        }
        // Run ends: add the run total to its row (emitted by the next thread in
        // this sub-chunk, and visible after the barrier above), or carry it.
        int nk = __shfl_down_sync(FULL_MASK, key, 1);
        if (lane == 31) nk = (warp + 1 < NW) ? sm.wfirst[warp + 1] : INT_MIN;
        if (tid == THREADS - 1) {
            sm.carry = acc;
            sm.next_row = i;
            sm.next_tile = j;
        } else if (nk != key) {
            Op::fix(y, mask, key, acc);
        }
        __syncthreads();
        carry = sm.carry;
        i0 = sm.next_row;
        j0 = sm.next_tile;
        __syncthreads();
    }
    if (tid == 0) {
        carries[blockIdx.x].row = i0;
        carries[blockIdx.x].val = carry;
    }
}

// Adds the CTA carries to their rows.  A run of CTAs ending in the same open
// row is summed in CTA order by the run's first thread.
template <class Op>
__global__ void carry_fixup_kernel(const CarryRec<Op>* __restrict__ carries, int grid, int nb,
                                   typename Op::Y* __restrict__ y,
                                   const typename Op::W* __restrict__ mask) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= grid) return;
    const int row = carries[c].row;
    if (row >= nb) return;
    if (c > 0 && carries[c - 1].row == row) return;
    typename Op::Acc tot = carries[c].val;
    for (int c2 = c + 1; c2 < grid && carries[c2].row == row; ++c2) Op::combine(tot, carries[c2].val);
    Op::fix(y, mask, row, tot);
}

template <class Op, int T, int THREADS, int ITEMS>
b2sr_status run_merge_spmv(const MatView& A, int grid, const Coord* d_starts, const void* x,
                           void* y, const void* mask, int accumulate, void* carries,
                           cudaStream_t s) {
    using W = typename Op::W;
    merge_spmv_kernel<Op, T, THREADS, ITEMS><<<grid, THREADS, 0, s>>>(
        A.rowptr, A.colind, reinterpret_cast<const W*>(A.tiles), A.nb, d_starts,
        reinterpret_cast<const typename Op::X*>(x), reinterpret_cast<typename Op::Y*>(y),
        reinterpret_cast<const W*>(mask), accumulate, reinterpret_cast<CarryRec<Op>*>(carries));
    B2SR_LAUNCH_CHECK();
    carry_fixup_kernel<Op><<<(grid + 127) / 128, 128, 0, s>>>(
        reinterpret_cast<const CarryRec<Op>*>(carries), grid, A.nb,
        reinterpret_cast<typename Op::Y*>(y), reinterpret_cast<const W*>(mask));
    B2SR_LAUNCH_CHECK();
    add_launch_count(2);
    return B2SR_SUCCESS;
}

// Dispatch over the supported launch shapes.
template <class Op, int T>
b2sr_status run_merge_shape(const MatView& A, const LaunchShape& sh, int grid,
                            const Coord* d_starts, const void* x, void* y, const void* mask,
                            int accumulate, void* carries, cudaStream_t s) {
    if (sh.threads == 256 && sh.items == 8)
        return run_merge_spmv<Op, T, 256, 8>(A, grid, d_starts, x, y, mask, accumulate, carries, s);
    if (sh.threads == 128 && sh.items == 16)
        return run_merge_spmv<Op, T, 128, 16>(A, grid, d_starts, x, y, mask, accumulate, carries, s);
    if (sh.threads == 256 && sh.items == 4)
        return run_merge_spmv<Op, T, 256, 4>(A, grid, d_starts, x, y, mask, accumulate, carries, s);
    return B2SR_ERR_NOT_SUPPORTED;
}

template <class Op, int T>
int max_ctas_per_sm(const LaunchShape& sh) {
    int n = 0;
    cudaError_t e = cudaErrorInvalidValue;
    if (sh.threads == 256 && sh.items == 8)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, merge_spmv_kernel<Op, T, 256, 8>, 256, 0);
    else if (sh.threads == 128 && sh.items == 16)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, merge_spmv_kernel<Op, T, 128, 16>, 128, 0);
    else if (sh.threads == 256 && sh.items == 4)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, merge_spmv_kernel<Op, T, 256, 4>, 256, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

}  // namespace b2sr
