// Merge-path B2SR multiply, shared by all variants.
//
// Work decomposition (merge-based SpMV, Merrill & Garland, SC'16, restated for
// B2SR): the work list is the merge of the nb tile-row ends with the nt tiles,
// nb + nt items.  A persistent grid splits it into equal shares (the start
// coordinate of every CTA is computed once per matrix by the partition
// kernel).  A CTA walks its share in sub-chunks of THREADS*ITEMS items:
//
//   1. stage the row ends the sub-chunk can reach in shared memory and find
//      every thread's merge-path start with a binary search there;
//   2. tile phase: lane q of the CTA takes tiles q, q+THREADS, ... of the
//      sub-chunk (coalesced colind/tile loads, independent x gathers, no
//      row-end divergence) and writes each tile's per-row partial ("part") to
//      shared memory;
//   3. merge phase: each thread consumes ITEMS consecutive items, adding the
//      parts of its tiles and writing a tile-row's T outputs at its row end;
//   4. tile-rows that span threads leave carries, combined by a segmented scan
//      in thread order; the last open row's carry moves to the next sub-chunk
//      and the CTA's final carry to a scratch array that the fix-up kernel
//      adds in CTA order.
// Every output is summed in one fixed order, so bin_full_full is bitwise
// reproducible and uses no float atomics (the reference's T < 32 kernels use
// atomicAdd, bsrbmv.cu:895,971,1036).
#pragma once

#include "b2sr_common.cuh"

namespace b2sr {

// ---- tile loads -------------------------------------------------------------------
// A tile as loaded (packed words: 4, 8, 32 or 128 bytes) and its rows widened
// to 32 bits (row r in rows[r]; bit T-1-c = column c).
template <int T> struct TileBits;

template <> struct TileBits<4> {
    uint32_t w;
    __device__ __forceinline__ void load(const uint8_t* tiles, int j) {
        w = __ldg(reinterpret_cast<const unsigned int*>(tiles) + j);
    }
    // Streaming load (evict-first): tile words are read once per multiply, so
    // they should not displace the gathered x lines in L1.
    __device__ __forceinline__ void load_stream(const uint8_t* tiles, int j) {
        w = __ldcs(reinterpret_cast<const unsigned int*>(tiles) + j);
    }
    __device__ __forceinline__ uint32_t row(int r) const { return (w >> (8 * r)) & 0xFu; }
};
template <> struct TileBits<8> {
    uint2 w;
    __device__ __forceinline__ void load(const uint8_t* tiles, int j) {
        w = __ldg(reinterpret_cast<const uint2*>(tiles) + j);
    }
    __device__ __forceinline__ void load_stream(const uint8_t* tiles, int j) {
        w = __ldcs(reinterpret_cast<const uint2*>(tiles) + j);
    }
    __device__ __forceinline__ uint32_t row(int r) const {
        return ((r < 4 ? w.x : w.y) >> (8 * (r & 3))) & 0xFFu;
    }
};
template <> struct TileBits<16> {
    uint4 a, b;
    __device__ __forceinline__ void load(const uint16_t* tiles, int j) {
        const uint4* p = reinterpret_cast<const uint4*>(tiles) + 2 * (size_t)j;
        a = __ldg(p);
        b = __ldg(p + 1);
    }
    __device__ __forceinline__ void load_stream(const uint16_t* tiles, int j) {
        const uint4* p = reinterpret_cast<const uint4*>(tiles) + 2 * (size_t)j;
        a = __ldcs(p);
        b = __ldcs(p + 1);
    }
    __device__ __forceinline__ uint32_t row(int r) const {
        const uint4& v = r < 8 ? a : b;
        const int k = (r & 7) >> 1;
        const uint32_t u = k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
        return (r & 1) ? (u >> 16) : (u & 0xFFFFu);
    }
};
template <> struct TileBits<32> {
    uint32_t w[32];
    __device__ __forceinline__ void load(const uint32_t* tiles, int j) {
        const uint4* p = reinterpret_cast<const uint4*>(tiles) + 8 * (size_t)j;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const uint4 v = __ldg(p + q);
            w[4 * q] = v.x;
            w[4 * q + 1] = v.y;
            w[4 * q + 2] = v.z;
            w[4 * q + 3] = v.w;
        }
    }
    __device__ __forceinline__ void load_stream(const uint32_t* tiles, int j) {
        const uint4* p = reinterpret_cast<const uint4*>(tiles) + 8 * (size_t)j;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const uint4 v = __ldcs(p + q);
            w[4 * q] = v.x;
            w[4 * q + 1] = v.y;
            w[4 * q + 2] = v.z;
            w[4 * q + 3] = v.w;
        }
    }
    __device__ __forceinline__ uint32_t row(int r) const { return w[r]; }
};

// Shared-memory slot of 16-byte unit s of the part array.  XOR-swizzling the
// low three bits with bits 3..5 keeps the tile phase (consecutive units per
// lane) conflict-free and spreads the merge phase's per-thread runs (unit
// stride ~ITEMS between lanes) over all bank groups.
__device__ __forceinline__ int swz(int s) { return s ^ ((s >> 3) & 7); }

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

template <int T>
__device__ __forceinline__ void store_row_f(float* __restrict__ y, int row, const float (&v)[T], int accumulate) {
    float4* p = reinterpret_cast<float4*>(y + (size_t)row * T);
#pragma unroll
    for (int q = 0; q < T / 4; ++q) {
        float4 o = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        if (accumulate) {
            const float4 old = p[q];
            o.x += old.x;
            o.y += old.y;
            o.z += old.z;
            o.w += old.w;
        }
        p[q] = o;
    }
}

// ---- variant ops ---------------------------------------------------------------------
// Each op defines:
//   Part / UNITS      per-tile partial, stored as UNITS 16-byte units in smem
//   make_part         tile phase: one tile -> its part (written to smem)
//   Acc / add_part    merge phase accumulator of one tile-row and its update
//   combine, shfl_up  carry arithmetic; emit / fix  output of a tile-row.
// Kernel arguments shared by all ops.
struct SpmvArgs {
    const int* rowptr;
    const int* colind;
    const void* tiles;
    const void* x;
    void* y;
    const void* mask;
    const Coord* starts;
    void* carries;
    int nb;
    int ncols;
    int accumulate;
};

// bin_full_full: FP32 x, FP32 y.  Within a tile the set bits of a row are
// added in ascending column order (the order of bmv32_bin_full_full,
// bsrbmv.cu:1063-1076); the tiles of a row are added in colind order inside a
// thread, threads are combined in thread order.
template <int T>
struct OpFullFull {
    using W = typename TileWord<T>::type;
    using Y = float;
    static constexpr int UNITS = T / 4;
    static constexpr bool XSCRATCH = T > 4;
    static constexpr int units(int tiles) { return tiles * UNITS; }
    struct Acc { float v[T]; };
    static __device__ __forceinline__ void zero(Acc& a) {
#pragma unroll
        for (int r = 0; r < T; ++r) a.v[r] = 0.0f;
    }
    // x segment of tile-column tc: vector loads for full segments, element
    // loads (bounded by ncols) for the last, partial one.
    static __device__ __forceinline__ void load_x(float (&xs)[T], const float* __restrict__ x, int tc,
                                                  int ncols) {
        const long long base = (long long)tc * T;
        if (base + T <= ncols) {
            const float4* p = reinterpret_cast<const float4*>(x + base);
#pragma unroll
            for (int q = 0; q < T / 4; ++q) {
                const float4 v = __ldg(p + q);
                xs[4 * q] = v.x;
                xs[4 * q + 1] = v.y;
                xs[4 * q + 2] = v.z;
                xs[4 * q + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int c = 0; c < T; ++c) xs[c] = (base + c < ncols) ? __ldg(x + base + c) : 0.0f;
        }
    }
    // Tile phase in three steps so a thread can keep several tiles' loads in
    // flight: raw tile words, then x segments, then the parts.
    static constexpr int BATCH = T <= 8 ? 4 : T == 16 ? 2 : 1;
    struct Raw { TileBits<T> bits; int tc; };
    struct XVal { float xs[T]; };
    static __device__ __forceinline__ void load_raw(Raw& r, const W* tiles, const int* colind, int j) {
        r.tc = __ldg(colind + j);
        r.bits.load(tiles, j);
    }
    static __device__ __forceinline__ void load_xval(XVal& v, const Raw& r, const SpmvArgs& a) {
        load_x(v.xs, static_cast<const float*>(a.x), r.tc, a.ncols);
    }
    static __device__ __forceinline__ void make_part(float4* parts, int q, const Raw& raw, const XVal& xv,
                                                     float* xscratch) {
        float s[T];
        if (T == 4) {
            // 16 predicated adds, no branches: a 4 x 4 tile has 16 cells.
#pragma unroll
            for (int r = 0; r < T; ++r) {
                float acc = 0.0f;
#pragma unroll
                for (int c = 0; c < T; ++c)
                    if (raw.bits.row(r) & (1u << (T - 1 - c))) acc += xv.xs[c];
                s[r] = acc;
            }
        } else {
            // Larger tiles are sparse: visit set bits only, reading the x
            // segment from this thread's smem scratch by column index.
#pragma unroll
            for (int c = 0; c < T; ++c) xscratch[c] = xv.xs[c];
#pragma unroll
            for (int r = 0; r < T; ++r) {
                uint32_t w = raw.bits.row(r);
                float acc = 0.0f;
                while (w) {
                    const int b = 31 - __clz(w);
                    acc += xscratch[T - 1 - b];
                    w &= ~(1u << b);
                }
                s[r] = acc;
            }
        }
#pragma unroll
        for (int u = 0; u < UNITS; ++u)
            parts[swz(q * UNITS + u)] = make_float4(s[4 * u], s[4 * u + 1], s[4 * u + 2], s[4 * u + 3]);
    }
    static __device__ __forceinline__ void add_part(Acc& a, const float4* parts, int q) {
#pragma unroll
        for (int u = 0; u < UNITS; ++u) {
            const float4 v = parts[swz(q * UNITS + u)];
            a.v[4 * u] += v.x;
            a.v[4 * u + 1] += v.y;
            a.v[4 * u + 2] += v.z;
            a.v[4 * u + 3] += v.w;
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
    static __device__ __forceinline__ void emit(const SpmvArgs& a, int row, const Acc& v) {
        store_row_f<T>(static_cast<float*>(a.y), row, v.v, a.accumulate);
    }
    static __device__ __forceinline__ void fix(const SpmvArgs& a, int row, const Acc& v) {
        store_row_f<T>(static_cast<float*>(a.y), row, v.v, 1);
    }
};

// bin_bin_full / bin_bin_count: bit x, count y (float or int32).  A tile's
// part holds the T row counts as bytes (a row of T <= 32 bits counts <= 32):
// 4 bytes for T = 4, 8 for T = 8, one or two 16-byte units for T = 16 / 32.
template <int T, typename YT>
struct OpCount {
    using W = typename TileWord<T>::type;
    using Y = YT;
    static constexpr bool XSCRATCH = false;
    static constexpr int NW32 = T / 4;  // packed 32-bit words per part
    static constexpr int units(int tiles) { return T == 4 ? (tiles + 3) / 4 : T == 8 ? (tiles + 1) / 2 : tiles * (T / 16); }
    struct Acc { int v[T]; };
    static __device__ __forceinline__ void zero(Acc& a) {
#pragma unroll
        for (int r = 0; r < T; ++r) a.v[r] = 0;
    }
    static constexpr int BATCH = T <= 8 ? 8 : T == 16 ? 4 : 2;
    struct Raw { TileBits<T> bits; int tc; };
    struct XVal { uint32_t xw; };
    static __device__ __forceinline__ void load_raw(Raw& r, const W* tiles, const int* colind, int j) {
        r.tc = __ldg(colind + j);
        r.bits.load(tiles, j);
    }
    static __device__ __forceinline__ void load_xval(XVal& v, const Raw& r, const SpmvArgs& a) {
        v.xw = __ldg(static_cast<const W*>(a.x) + r.tc);
    }
    static __device__ __forceinline__ void make_part(float4* parts, int q, const Raw& raw, const XVal& xv,
                                                     float*) {
        const uint32_t xw = xv.xw;
        uint32_t packed[NW32];
#pragma unroll
        for (int k = 0; k < NW32; ++k) packed[k] = 0;
#pragma unroll
        for (int r = 0; r < T; ++r) packed[r / 4] |= (uint32_t)__popc(raw.bits.row(r) & xw) << (8 * (r % 4));
        if constexpr (T == 4) {
            reinterpret_cast<uint32_t*>(parts)[swz(q / 4) * 4 + q % 4] = packed[0];
        } else if constexpr (T == 8) {
            reinterpret_cast<uint2*>(parts)[swz(q / 2) * 2 + q % 2] = make_uint2(packed[0], packed[1]);
        } else {
#pragma unroll
            for (int u = 0; u < T / 16; ++u)
                reinterpret_cast<uint4*>(parts)[swz(q * (T / 16) + u)] =
                    make_uint4(packed[4 * u], packed[4 * u + 1], packed[4 * u + 2], packed[4 * u + 3]);
        }
    }
    static __device__ __forceinline__ void add_part(Acc& a, const float4* parts, int q) {
        uint32_t packed[NW32];
        if constexpr (T == 4) {
            packed[0] = reinterpret_cast<const uint32_t*>(parts)[swz(q / 4) * 4 + q % 4];
        } else if constexpr (T == 8) {
            const uint2 v = reinterpret_cast<const uint2*>(parts)[swz(q / 2) * 2 + q % 2];
            packed[0] = v.x;
            packed[1] = v.y;
        } else {
#pragma unroll
            for (int u = 0; u < T / 16; ++u) {
                const uint4 v = reinterpret_cast<const uint4*>(parts)[swz(q * (T / 16) + u)];
                packed[4 * u] = v.x;
                packed[4 * u + 1] = v.y;
                packed[4 * u + 2] = v.z;
                packed[4 * u + 3] = v.w;
            }
        }
#pragma unroll
        for (int r = 0; r < T; ++r) a.v[r] += (packed[r / 4] >> (8 * (r % 4))) & 0xFFu;
    }
    static __device__ __forceinline__ void combine(Acc& a, const Acc& b) {
#pragma unroll
        for (int r = 0; r < T; ++r) a.v[r] += b.v[r];
    }
    static __device__ __forceinline__ void shfl_up(Acc& out, const Acc& a, int o) {
#pragma unroll
        for (int r = 0; r < T; ++r) out.v[r] = __shfl_up_sync(FULL_MASK, a.v[r], o);
    }
    static __device__ __forceinline__ void emit(const SpmvArgs& a, int row, const Acc& v) {
        Y o[T];
#pragma unroll
        for (int r = 0; r < T; ++r) o[r] = (Y)v.v[r];
        store_row<T, Y>(static_cast<Y*>(a.y), row, o, a.accumulate);
    }
    static __device__ __forceinline__ void fix(const SpmvArgs& a, int row, const Acc& v) {
        Y o[T];
#pragma unroll
        for (int r = 0; r < T; ++r) o[r] = (Y)v.v[r];
        store_row<T, Y>(static_cast<Y*>(a.y), row, o, 1);
    }
};

// bin_bin_bin: bit x, bit y; row r of the output word is set when any tile of
// the tile-row shares a bit between its row r and the x word (the reference's
// popc(A & x) > 0 vote, bsrbmv.cu:300-309).  MASKED: y = result AND NOT mask,
// overwriting (bsrbmv.cu:1113-1118).  A tile's part is its T-bit row mask.
template <int T, bool MASKED>
struct OpBits {
    using W = typename TileWord<T>::type;
    using Y = W;
    static constexpr bool XSCRATCH = false;
    static constexpr int units(int tiles) { return (tiles + 3) / 4; }  // 4-byte parts, 4 per unit
    struct Acc { uint32_t m; };
    static __device__ __forceinline__ void zero(Acc& a) { a.m = 0; }
    static constexpr int BATCH = T <= 8 ? 8 : T == 16 ? 4 : 2;
    struct Raw { TileBits<T> bits; int tc; };
    struct XVal { uint32_t xw; };
    static __device__ __forceinline__ void load_raw(Raw& r, const W* tiles, const int* colind, int j) {
        r.tc = __ldg(colind + j);
        r.bits.load(tiles, j);
    }
    static __device__ __forceinline__ void load_xval(XVal& v, const Raw& r, const SpmvArgs& a) {
        v.xw = __ldg(static_cast<const W*>(a.x) + r.tc);
    }
    static __device__ __forceinline__ void make_part(float4* parts, int q, const Raw& raw, const XVal& xv,
                                                     float*) {
        const uint32_t xw = xv.xw;
        uint32_t m = 0;
#pragma unroll
        for (int r = 0; r < T; ++r) m |= ((raw.bits.row(r) & xw) != 0u ? 1u : 0u) << (T - 1 - r);
        reinterpret_cast<uint32_t*>(parts)[swz(q / 4) * 4 + q % 4] = m;
    }
    static __device__ __forceinline__ void add_part(Acc& a, const float4* parts, int q) {
        a.m |= reinterpret_cast<const uint32_t*>(parts)[swz(q / 4) * 4 + q % 4];
    }
    static __device__ __forceinline__ void combine(Acc& a, const Acc& b) { a.m |= b.m; }
    static __device__ __forceinline__ void shfl_up(Acc& out, const Acc& a, int o) {
        out.m = __shfl_up_sync(FULL_MASK, a.m, o);
    }
    static __device__ __forceinline__ void emit(const SpmvArgs& a, int row, const Acc& v) {
        W* y = static_cast<W*>(a.y);
        if (MASKED) {
            y[row] = (W)(v.m & ~(uint32_t)static_cast<const W*>(a.mask)[row]);
        } else {
            y[row] = (W)(a.accumulate ? ((uint32_t)y[row] | v.m) : v.m);
        }
    }
    static __device__ __forceinline__ void fix(const SpmvArgs& a, int row, const Acc& v) {
        W* y = static_cast<W*>(a.y);
        const uint32_t add = MASKED ? (v.m & ~(uint32_t)static_cast<const W*>(a.mask)[row]) : v.m;
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
// spaced rows per round.  The predicate "row x has ended before tile d-x-1"
// (rowptr[x+1] <= d-x-1) is true then false along x; the coordinate is the
// first x where it is false.
__global__ void partition_kernel(const int* __restrict__ rowptr, int nb, int grid,
                                 Coord* __restrict__ starts);

// Shared memory of the multiply kernel: [row ends | parts | x scratch].
template <class Op, int T, int THREADS, int ITEMS>
struct MergeLayout {
    static constexpr int IPC = THREADS * ITEMS;
    static constexpr int ROWEND_BYTES = ((IPC + 1) * 4 + 15) / 16 * 16;
    static constexpr int PART_BYTES = Op::units(IPC) * 16;
    static constexpr int XS_BYTES = Op::XSCRATCH ? THREADS * T * 4 : 0;
    static constexpr int BYTES = ROWEND_BYTES + PART_BYTES + XS_BYTES;
};

template <class Op>
struct BlockScratch {
    int wkey[32];
    int wfirst[32];
    typename Op::Acc wacc[32];
    int next_row, next_tile, end_row, end_tile;
    typename Op::Acc carry;
};

// ---- the multiply kernel ----------------------------------------------------------------------
template <class Op, int T, int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS)
merge_spmv_kernel(SpmvArgs a) {
    using Acc = typename Op::Acc;
    using W = typename Op::W;
    using L = MergeLayout<Op, T, THREADS, ITEMS>;
    constexpr int IPC = L::IPC;
    constexpr int NW = THREADS / 32;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ BlockScratch<Op> bs;
    int* rowend = reinterpret_cast<int*>(smem);
    float4* parts = reinterpret_cast<float4*>(smem + L::ROWEND_BYTES);
    float* xscratch = reinterpret_cast<float*>(smem + L::ROWEND_BYTES + L::PART_BYTES) +
                      (L::XS_BYTES ? threadIdx.x * T : 0);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb = a.nb;
    const int* __restrict__ rowptr = a.rowptr;
    const int* __restrict__ colind = a.colind;
    const W* __restrict__ tiles = static_cast<const W*>(a.tiles);
    const int nt = rowptr[nb];
    const Coord beg = a.starts[blockIdx.x];
    const Coord end = a.starts[blockIdx.x + 1];
    const long long d_end = (long long)end.row + end.tile;
    int i0 = beg.row, j0 = beg.tile;
    Acc carry;
    Op::zero(carry);

    while ((long long)i0 + j0 < d_end) {
        const int n_items = (int)min((long long)IPC, d_end - ((long long)i0 + j0));
        // 1. row ends of the rows this sub-chunk can reach (at most n_items)
        for (int k = tid; k <= n_items; k += THREADS) {
            const int r = i0 + k;
            rowend[k] = r < nb ? __ldg(rowptr + r + 1) : nt;
        }
        __syncthreads();
        // merge-path search on the staged row ends: rows consumed at item rd,
        // searched within [lo, hi] (hi bounded by the rows of this sub-chunk
        // once the sub-chunk end is known)
        auto search = [&](int rd, int lo, int hi) {
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (rowend[mid] <= j0 + rd - mid - 1) lo = mid + 1;
                else hi = mid;
            }
            return lo;
        };
        if (tid == 0) {
            const int xe = search(n_items, max(0, n_items - (nt - j0)), min(n_items, nb - i0));
            bs.end_row = xe;
            bs.end_tile = j0 + n_items - xe;
        }
        __syncthreads();
        const int x_end = bs.end_row;
        const int ntile = bs.end_tile - j0;

        // 2. tile phase: parts of tiles [j0, j0 + ntile), BATCH tiles per
        //    thread at a time with all their loads in flight together.
        for (int q0 = 0; q0 < ntile; q0 += THREADS * Op::BATCH) {
            typename Op::Raw raw[Op::BATCH];
            typename Op::XVal xv[Op::BATCH];
#pragma unroll
            for (int u = 0; u < Op::BATCH; ++u) {
                const int q = q0 + u * THREADS + tid;
                if (q < ntile) Op::load_raw(raw[u], tiles, colind, j0 + q);
            }
#pragma unroll
            for (int u = 0; u < Op::BATCH; ++u) {
                const int q = q0 + u * THREADS + tid;
                if (q < ntile) Op::load_xval(xv[u], raw[u], a);
            }
#pragma unroll
            for (int u = 0; u < Op::BATCH; ++u) {
                const int q = q0 + u * THREADS + tid;
                if (q < ntile) Op::make_part(parts, q, raw[u], xv[u], xscratch);
            }
        }
        __syncthreads();

        // this thread's start coordinate
        const int rd = min(tid * ITEMS, n_items);
        const int x0 = search(rd, max(0, rd - ntile), min(rd, x_end));

        // 3. merge phase
        int i = i0 + x0, j = j0 + rd - x0;
        const int my_items = min(ITEMS, n_items - rd);
        Acc acc;
        if (tid == 0) acc = carry;
        else Op::zero(acc);
        for (int k = 0; k < my_items; ++k) {
            if (j < rowend[i - i0]) {
                Op::add_part(acc, parts, j - j0);
                ++j;
            } else {
                Op::emit(a, i, acc);
                Op::zero(acc);
                ++i;
            }
        }

        // 4. segmented inclusive scan of the carries keyed by the open row;
        //    keys are non-decreasing in thread order.
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
            bs.wkey[warp] = key;
            bs.wfirst[warp] = first_key;
            bs.wacc[warp] = acc;
        }
        __syncthreads();
        if (warp > 0 && key == first_key) {
            Acc pre;
            Op::zero(pre);
            bool any = false;
            for (int w2 = warp - 1; w2 >= 0; --w2) {
                if (bs.wkey[w2] != key) break;
                Acc t = bs.wacc[w2];
                Op::combine(t, pre);
                pre = t;
                any = true;
                if (bs.wfirst[w2] != key) break;
            }
            if (any) {
                Op::combine(pre, acc);
                acc = pre;
            }
        }
        // Run ends add their run total to the row (emitted by the next thread
        // in this sub-chunk, visible after the barrier above) or carry it.
        int nk = __shfl_down_sync(FULL_MASK, key, 1);
        if (lane == 31) nk = (warp + 1 < NW) ? bs.wfirst[warp + 1] : INT_MIN;
        if (tid == THREADS - 1) {
            bs.carry = acc;
            bs.next_row = i;
            bs.next_tile = j;
        } else if (nk != key) {
            Op::fix(a, key, acc);
        }
        __syncthreads();
        carry = bs.carry;
        i0 = bs.next_row;
        j0 = bs.next_tile;
    }
    if (tid == 0) {
        CarryRec<Op>* carries = static_cast<CarryRec<Op>*>(a.carries);
        carries[blockIdx.x].row = i0;
        carries[blockIdx.x].val = carry;
    }
}

// Adds the CTA carries to their rows.  A run of CTAs ending in the same open
// row is summed in CTA order by the run's first thread.
template <class Op>
__global__ void carry_fixup_kernel(SpmvArgs a, int grid) {
    griddep_wait();  // launched behind the merge-path kernel: its carries
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= grid) return;
    const CarryRec<Op>* carries = static_cast<const CarryRec<Op>*>(a.carries);
    const int row = carries[c].row;
    if (row >= a.nb) return;
    if (c > 0 && carries[c - 1].row == row) return;
    typename Op::Acc tot = carries[c].val;
    for (int c2 = c + 1; c2 < grid && carries[c2].row == row; ++c2) Op::combine(tot, carries[c2].val);
    Op::fix(a, row, tot);
}

// The dynamic shared-memory limit is a per-device attribute of the kernel, so
// it is set on every launch (a host-side call, no synchronization): a value
// cached once per process would not cover a second device.
template <class Op, int T, int THREADS, int ITEMS>
cudaError_t prepare_kernel() {
    return cudaFuncSetAttribute(merge_spmv_kernel<Op, T, THREADS, ITEMS>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                MergeLayout<Op, T, THREADS, ITEMS>::BYTES);
}

template <class Op, int T, int THREADS, int ITEMS>
b2sr_status run_merge_spmv(const SpmvArgs& args, int grid, cudaStream_t s) {
    cudaError_t e = prepare_kernel<Op, T, THREADS, ITEMS>();
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return B2SR_ERR_CUDA;
    }
    kernel_timer_mark(s, true);
    merge_spmv_kernel<Op, T, THREADS, ITEMS>
        <<<grid, THREADS, MergeLayout<Op, T, THREADS, ITEMS>::BYTES, s>>>(args);
    kernel_timer_mark(s, false);
    B2SR_LAUNCH_CHECK();
    B2SR_CUDA_TRY(launch_dependent(carry_fixup_kernel<Op>, (unsigned)((grid + 127) / 128), 128u, s, args, grid));
    add_launch_count(2);
    return B2SR_SUCCESS;
}

// Supported launch shapes (threads, items per thread).
#define B2SR_FOR_EACH_SHAPE(X) X(256, 8) X(256, 4) X(128, 16) X(128, 8) X(128, 4)

template <class Op, int T>
b2sr_status run_merge_shape(const SpmvArgs& args, const LaunchShape& sh, int grid, cudaStream_t s) {
#define B2SR_TRY_SHAPE(TH, IT) \
    if (sh.threads == TH && sh.items == IT) return run_merge_spmv<Op, T, TH, IT>(args, grid, s);
    B2SR_FOR_EACH_SHAPE(B2SR_TRY_SHAPE)
#undef B2SR_TRY_SHAPE
    return B2SR_ERR_NOT_SUPPORTED;
}

template <class Op, int T>
int max_ctas_per_sm(const LaunchShape& sh) {
    int n = 0;
    cudaError_t e = cudaErrorInvalidValue;
#define B2SR_OCC_SHAPE(TH, IT)                                                                    \
    if (sh.threads == TH && sh.items == IT) {                                                     \
        e = prepare_kernel<Op, T, TH, IT>();                                                      \
        if (e == cudaSuccess)                                                                     \
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(                                    \
                &n, merge_spmv_kernel<Op, T, TH, IT>, TH, MergeLayout<Op, T, TH, IT>::BYTES);      \
    }
    B2SR_FOR_EACH_SHAPE(B2SR_OCC_SHAPE)
#undef B2SR_OCC_SHAPE
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

}  // namespace b2sr
