// B2SR x dense multiply on the merge path: Y = A . X with X [ncols, k] and
// Y [nb*T, k] row-major (FP32 or FP64), the bin_full_full variant on feature
// blocks.  The library runs the row-task kernel (b2sr_spmm_rows.cu) by
// default; this one runs when a matrix's bin_full_full launch option sets
// algorithm = merge.
//
// Decomposition: the merge path of tile-row ends and tiles is cut into
// chunks of CHUNK items whose start coordinates are computed on the device;
// warps take chunks from a work queue (an atomic counter).  Inside a warp all
// lanes walk the same tiles and set bits (warp-uniform control flow) and lane
// l owns columns [l*VEC, l*VEC + VEC) of a KC = 32*VEC column block, so each
// X row of a set bit is fetched with one coalesced 128/256/512-byte load.  A
// chunk that ends inside a tile-row stores its partial rows as a carry; the
// fix-up kernel adds the carries of a row in chunk order, so the result does
// not depend on which warp ran which chunk.  k wider than KC is processed in
// column blocks.
#include <algorithm>

#include "b2sr_spmv_impl.cuh"

namespace b2sr {

template <typename V, int VEC> struct VecOf;
template <> struct VecOf<float, 1> { using type = float; };
template <> struct VecOf<float, 2> { using type = float2; };
template <> struct VecOf<float, 4> { using type = float4; };
template <> struct VecOf<double, 1> { using type = double; };
template <> struct VecOf<double, 2> { using type = double2; };

template <typename V, int VEC>
__device__ __forceinline__ void load_vec(V (&out)[VEC], const V* p, bool aligned_full, int nvalid) {
    if (aligned_full) {
        using VT = typename VecOf<V, VEC>::type;
        const VT v = __ldg(reinterpret_cast<const VT*>(p));
        const V* e = reinterpret_cast<const V*>(&v);
#pragma unroll
        for (int i = 0; i < VEC; ++i) out[i] = e[i];
    } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i) out[i] = i < nvalid ? __ldg(p + i) : V(0);
    }
}

template <typename V, int VEC>
__device__ __forceinline__ void store_vec(V* p, const V (&v)[VEC], bool aligned_full, int nvalid,
                                          bool accumulate) {
    if (aligned_full) {
        using VT = typename VecOf<V, VEC>::type;
        VT* q = reinterpret_cast<VT*>(p);
        VT o;
        V* e = reinterpret_cast<V*>(&o);
        if (accumulate) {
            const VT old = *q;
            const V* oe = reinterpret_cast<const V*>(&old);
#pragma unroll
            for (int i = 0; i < VEC; ++i) e[i] = oe[i] + v[i];
        } else {
#pragma unroll
            for (int i = 0; i < VEC; ++i) e[i] = v[i];
        }
        *q = o;
    } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i)
            if (i < nvalid) p[i] = accumulate ? p[i] + v[i] : v[i];
    }
}

template <typename V>
struct SpmmArgs {
    const int* rowptr;
    const int* colind;
    const void* tiles;
    const V* X;
    V* Y;
    long long ldx, ldy;
    int k;        // total columns
    int kc0;      // first column of this column block
    const Coord* starts;
    int nchunks;
    int* counter;
    V* carry_vals;   // nchunks x T x KC
    int* carry_rows;  // nchunks
    int nb;
    int accumulate;
    int vec_ok;       // X, Y, ldx, ldy allow VEC-wide vector access
};

// acc[r] += v for a warp-uniform row index r (a uniform branch, no local memory).
template <int T, int VEC, typename V>
__device__ __forceinline__ void add_row(V (&acc)[T][VEC], int r, const V (&v)[VEC]) {
#pragma unroll
    for (int rr = 0; rr < T; ++rr)
        if (rr == r) {
#pragma unroll
            for (int e = 0; e < VEC; ++e) acc[rr][e] += v[e];
        }
}

// Adds tile j's contributions.  Set bits are taken two at a time so two X-row
// loads are in flight before either is added.  For T = 4/8 the packed tile
// word is walked directly (row = bit / 8); for T = 16/32 rows are walked in
// order with their bits.
template <int T, int VEC, typename V>
__device__ __forceinline__ void spmm_tile(V (&acc)[T][VEC], const TileBits<T>& tb, long long xbase,
                                          const SpmmArgs<V>& a, int col, bool full, int nvalid) {
    auto xrow = [&](int c) { return a.X + (xbase + c) * a.ldx + col; };
    if constexpr (T == 4 || T == 8) {
        // T = 4: 4 bytes, row r = byte r, column c at bit 8r + 3 - c (low nibble)
        // T = 8: 8 bytes, row r = byte r, column c at bit 8r + 7 - c
        unsigned long long w;
        if constexpr (T == 4) w = tb.w;
        else w = ((unsigned long long)tb.w.y << 32) | tb.w.x;
        while (w) {
            const int p1 = 63 - __clzll(w);
            w ^= 1ull << p1;
            V x1[VEC];
            if (w) {
                const int p2 = 63 - __clzll(w);
                w ^= 1ull << p2;
                V x2[VEC];
                load_vec<V, VEC>(x1, xrow(T - 1 - (p1 & 7)), full, nvalid);
                load_vec<V, VEC>(x2, xrow(T - 1 - (p2 & 7)), full, nvalid);
                add_row<T, VEC, V>(acc, p1 >> 3, x1);
                add_row<T, VEC, V>(acc, p2 >> 3, x2);
            } else {
                load_vec<V, VEC>(x1, xrow(T - 1 - (p1 & 7)), full, nvalid);
                add_row<T, VEC, V>(acc, p1 >> 3, x1);
            }
        }
    } else {
#pragma unroll
        for (int r = 0; r < T; ++r) {
            uint32_t w = tb.row(r);
            while (w) {
                const int b1 = 31 - __clz(w);
                w ^= 1u << b1;
                V x1[VEC];
                if (w) {
                    const int b2 = 31 - __clz(w);
                    w ^= 1u << b2;
                    V x2[VEC];
                    load_vec<V, VEC>(x1, xrow(T - 1 - b1), full, nvalid);
                    load_vec<V, VEC>(x2, xrow(T - 1 - b2), full, nvalid);
#pragma unroll
                    for (int e = 0; e < VEC; ++e) {
                        acc[r][e] += x1[e];
                        acc[r][e] += x2[e];
                    }
                } else {
                    load_vec<V, VEC>(x1, xrow(T - 1 - b1), full, nvalid);
#pragma unroll
                    for (int e = 0; e < VEC; ++e) acc[r][e] += x1[e];
                }
            }
        }
    }
}

template <int T, int VEC, typename V>
__global__ void __launch_bounds__(256)
spmm_kernel(SpmmArgs<V> a) {
    using W = typename TileWord<T>::type;
    constexpr int KC = 32 * VEC;
    const int lane = threadIdx.x & 31;
    const int col = a.kc0 + lane * VEC;
    const int nvalid = max(0, min(VEC, a.k - col));
    const bool full = a.vec_ok && nvalid == VEC;
    const W* tiles = static_cast<const W*>(a.tiles);
    const int nt = a.rowptr[a.nb];
    while (true) {
        int c = 0;
        if (lane == 0) c = atomicAdd(a.counter, 1);
        c = __shfl_sync(FULL_MASK, c, 0);
        if (c >= a.nchunks) break;
        const Coord beg = a.starts[c], end = a.starts[c + 1];
        int i = beg.row, j = beg.tile;
        const long long d_end = (long long)end.row + end.tile;
        V acc[T][VEC];
#pragma unroll
        for (int r = 0; r < T; ++r)
#pragma unroll
            for (int v = 0; v < VEC; ++v) acc[r][v] = V(0);
        int row_end = i < a.nb ? __ldg(a.rowptr + i + 1) : nt;
        while ((long long)i + j < d_end) {
            if (j < row_end) {
                TileBits<T> tb;
                tb.load(tiles, j);
                spmm_tile<T, VEC, V>(acc, tb, (long long)__ldg(a.colind + j) * T, a, col, full, nvalid);
                ++j;
            } else {
#pragma unroll
                for (int r = 0; r < T; ++r) {
                    if (nvalid > 0)
                        store_vec<V, VEC>(a.Y + ((long long)i * T + r) * a.ldy + col, acc[r], full, nvalid,
                                          a.accumulate != 0);
#pragma unroll
                    for (int v = 0; v < VEC; ++v) acc[r][v] = V(0);
                }
                ++i;
                row_end = i < a.nb ? __ldg(a.rowptr + i + 1) : nt;
            }
        }
        // carry: the open row's partial (zero when the chunk ended on a row end)
        if (lane == 0) a.carry_rows[c] = i;
        V* cv = a.carry_vals + (long long)c * T * KC + lane * VEC;
#pragma unroll
        for (int r = 0; r < T; ++r)
#pragma unroll
            for (int v = 0; v < VEC; ++v) cv[r * KC + v] = acc[r][v];
    }
}

// One warp per chunk: the first chunk of a run ending in the same open row
// adds the run's carries to that row, in chunk order.
template <int T, int VEC, typename V>
__global__ void spmm_fixup_kernel(SpmmArgs<V> a) {
    griddep_wait();  // launched behind the main kernel: its carries
    constexpr int KC = 32 * VEC;
    const int lane = threadIdx.x & 31;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= a.nchunks) return;
    const int row = a.carry_rows[c];
    if (row >= a.nb || (c > 0 && a.carry_rows[c - 1] == row)) return;
    const int col = a.kc0 + lane * VEC;
    const int nvalid = max(0, min(VEC, a.k - col));
    V tot[T][VEC];
#pragma unroll
    for (int r = 0; r < T; ++r)
#pragma unroll
        for (int v = 0; v < VEC; ++v) tot[r][v] = V(0);
    for (int c2 = c; c2 < a.nchunks && a.carry_rows[c2] == row; ++c2) {
        const V* cv = a.carry_vals + (long long)c2 * T * KC + lane * VEC;
#pragma unroll
        for (int r = 0; r < T; ++r)
#pragma unroll
            for (int v = 0; v < VEC; ++v) tot[r][v] += cv[r * KC + v];
    }
    if (nvalid == 0) return;
#pragma unroll
    for (int r = 0; r < T; ++r) store_vec<V, VEC>(a.Y + ((long long)row * T + r) * a.ldy + col, tot[r], false, nvalid, true);
}

template <int T, int VEC, typename V>
static b2sr_status run_spmm(SpmmArgs<V> a, int grid_warps, cudaStream_t s) {
    const int threads = 256;
    const int blocks = (grid_warps * 32 + threads - 1) / threads;
    cudaError_t e = cudaMemsetAsync(a.counter, 0, sizeof(int), s);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return B2SR_ERR_CUDA;
    }
    kernel_timer_mark(s, true);
    spmm_kernel<T, VEC, V><<<blocks, threads, 0, s>>>(a);
    kernel_timer_mark(s, false);
    B2SR_LAUNCH_CHECK();
    B2SR_CUDA_TRY(launch_dependent(spmm_fixup_kernel<T, VEC, V>, (unsigned)((a.nchunks * 32 + 255) / 256), 256u, s, a));
    add_launch_count(2);
    return B2SR_SUCCESS;
}

// Columns per lane: the narrowest column block (32*VEC) that covers k, with
// at most 32 registers of accumulators (T*VEC values: 32 FP32, 16 FP64) per
// lane and 16-byte vectors.  Every (T, VEC) this gives is instantiated below.
int spmm_vec(int T, int elem_bytes, int k) {
    const int max_vec = std::min(16 / elem_bytes, std::max(1, 32 / T * 4 / elem_bytes));
    int vec = 1;
    while (vec < max_vec && 32 * vec < k) vec *= 2;
    return vec;
}

template <typename V>
b2sr_status spmm_launch(const MatView& A, const V* X, long long ldx, V* Y, long long ldy, int k,
                        int accumulate, const Coord* starts, int nchunks, void* scratch, int grid_warps,
                        cudaStream_t s) {
    const int T = A.T;
    const int vec = spmm_vec(T, (int)sizeof(V), k);
    const int KC = 32 * vec;
    SpmmArgs<V> a;
    a.rowptr = A.rowptr;
    a.colind = A.colind;
    a.tiles = A.tiles;
    a.X = X;
    a.Y = Y;
    a.ldx = ldx;
    a.ldy = ldy;
    a.k = k;
    a.starts = starts;
    a.nchunks = nchunks;
    a.counter = static_cast<int*>(scratch);
    a.carry_rows = static_cast<int*>(scratch) + 4;
    size_t off = ((size_t)(nchunks + 4) * sizeof(int) + 255) / 256 * 256;
    a.carry_vals = reinterpret_cast<V*>(static_cast<char*>(scratch) + off);
    a.nb = A.nb;
    a.accumulate = accumulate;
    const size_t vb = sizeof(V) * vec;
    a.vec_ok = ((uintptr_t)X % vb == 0) && ((uintptr_t)Y % vb == 0) && (ldx % vec == 0) && (ldy % vec == 0);
    for (int kc0 = 0; kc0 < k; kc0 += KC) {
        a.kc0 = kc0;
        b2sr_status st = B2SR_ERR_INVALID_VALUE;
#define B2SR_SPMM_CASE(TT, VV) \
        if (T == TT && vec == VV) st = run_spmm<TT, VV, V>(a, grid_warps, s);
        if constexpr (sizeof(V) == 4) {
            B2SR_SPMM_CASE(4, 1) B2SR_SPMM_CASE(4, 2) B2SR_SPMM_CASE(4, 4)
            B2SR_SPMM_CASE(8, 1) B2SR_SPMM_CASE(8, 2) B2SR_SPMM_CASE(8, 4)
            B2SR_SPMM_CASE(16, 1) B2SR_SPMM_CASE(16, 2) B2SR_SPMM_CASE(32, 1)
        } else {
            B2SR_SPMM_CASE(4, 1) B2SR_SPMM_CASE(4, 2) B2SR_SPMM_CASE(8, 1) B2SR_SPMM_CASE(8, 2)
            B2SR_SPMM_CASE(16, 1) B2SR_SPMM_CASE(32, 1)
        }
#undef B2SR_SPMM_CASE
        if (st != B2SR_SUCCESS) return st;
    }
    return B2SR_SUCCESS;
}

size_t spmm_scratch_bytes(int T, int elem_bytes, int nchunks, int k) {
    const int vec = spmm_vec(T, elem_bytes, k);
    const size_t off = ((size_t)(nchunks + 4) * sizeof(int) + 255) / 256 * 256;
    return off + (size_t)nchunks * T * 32 * vec * elem_bytes;
}

int spmm_grid_warps(int num_sms) { return num_sms * 48; }

template b2sr_status spmm_launch<float>(const MatView&, const float*, long long, float*, long long, int, int,
                                        const Coord*, int, void*, int, cudaStream_t);
template b2sr_status spmm_launch<double>(const MatView&, const double*, long long, double*, long long, int,
                                         int, const Coord*, int, void*, int, cudaStream_t);

}  // namespace b2sr
