// Row-binned bin_full_full multiply: the fast path of y = A.x for packed
// matrices (the merge-path kernel in b2sr_spmv_impl.cuh serves the other
// variants and the reference-compatible shims).
//
// Plan (once per matrix, built on the host from rowptr): every tile-row is
// put in a bin by its tile count m; a bin fixes the group size G (lanes per
// tile-row) so that each lane handles at most U tiles:
//     m <= U -> G = 1,  m <= 2U -> 2,  ... ,  m <= 16U -> 16,  else G = 32.
// Tile-rows longer than 32*U tiles are cut into segments of 32*U tiles.
// A task is (row, first tile, end tile, out): out = -1 writes y directly,
// out >= 0 writes a segment partial that the fix-up kernel adds in segment
// order.  Tasks are stored bin by bin; a warp takes 32/G tasks of one bin.
//
// Kernel: each lane loads the colind/tile words of its (at most U) tiles,
// then their x segments, all in flight together, and adds the tiles' row
// sums into T register accumulators.  The group's G partial vectors are
// combined by a butterfly reduce-scatter of log2(G) shuffle steps, after
// which each lane holds T/G finished rows (or one row shared by G/T lanes).
// No shared memory, no block barriers, no atomics; the summation order is
// fixed, so the result is bitwise reproducible.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <vector>

#include "b2sr_spmv_impl.cuh"

namespace b2sr {

constexpr int RB_BINS = 6;  // G = 1, 2, 4, 8, 16, 32

template <int T> struct RowBinU { static constexpr int value = T <= 8 ? 4 : T == 16 ? 2 : 1; };
// Tiles per lane of the bit-vector kernel's long-row tasks (a full warp
// each, one step): 8 at T = 4, where its tiles need few registers.  The FP32 /
// OR kernel keeps RowBinU there too (its registers buy occupancy), so the two
// kernels have separate plans.
constexpr int rb_long_u(int T) { return T == 4 ? 8 : T == 8 ? 4 : T == 16 ? 2 : 1; }
template <int T, int G> struct RowBinTaskU {
    static constexpr int value = G == 32 ? rb_long_u(T) : RowBinU<T>::value;
};

struct RowBinArgs {
    const int* colind;
    const void* tiles;
    const void* x;
    void* y;
    const void* mask;   // OR semirings: y = result AND NOT mask (nullptr: no mask)
    const int4* tasks;  // (row, tile begin, tile end, out)
    void* partials;     // out slots x T values
    int task_off[RB_BINS + 1];
    int warp_off[RB_BINS + 1];
    int ncols;
    int accumulate;
    cudaTextureObject_t xtex;  // 0: x segments through ld.global; else uint4 texels of x
};

// Semirings of the row-binned kernel: FP32 (+) for bin_full_full, and
// bitwise OR over 32- or 64-bit words for the multi-frontier Boolean product
// (one bit per frontier, as many frontiers as word bits).
// `clear(v, m)` applies a mask word (OR semirings only: v AND NOT m).
struct SemSumF32 {
    using V = float;
    static __device__ __forceinline__ V zero() { return 0.0f; }
    static __device__ __forceinline__ V add(V a, V b) { return a + b; }
    static __device__ __forceinline__ V clear(V a, V) { return a; }
};
struct SemOrU32 {
    using V = uint32_t;
    static __device__ __forceinline__ V zero() { return 0u; }
    static __device__ __forceinline__ V add(V a, V b) { return a | b; }
    static __device__ __forceinline__ V clear(V a, V m) { return a & ~m; }
};
struct SemOrU64 {
    using V = unsigned long long;
    static __device__ __forceinline__ V zero() { return 0ull; }
    static __device__ __forceinline__ V add(V a, V b) { return a | b; }
    static __device__ __forceinline__ V clear(V a, V m) { return a & ~m; }
};

// Set columns of an FP32 tile gathered at once before the adds in the
// sparse-column form; a tile with more takes the rest in a loop.  On R-MAT
// scale 20, 1.6% / 4.2% / 8.3% / 8.4% of the tiles have more than 2 / 2 / 2 /
// 3 set columns at T = 4 / 8 / 16 / 32 (K = 3 at T = 16 measured slower).
template <int T> struct SparseColsK { static constexpr int value = T == 32 ? 3 : 2; };

// One tile of a lane: its packed rows, tile-column, and the x segment of
// that tile-column.  add_to folds the tile's rows into acc: every set bit
// (r, c) adds x[c] to row r, columns ascending (T = 4: 16 predicated adds;
// larger FP32 tiles sum each row first).
//
// FP32 tiles can take the sparse-column form instead (SparseColTile, the
// default at T = 16 and 32, launch option gather = 3 at any T): only the x
// elements of the tile's set columns are loaded, and each row adds only
// those, so a tile costs O(T x set columns) rather than T^2 predicated adds
// and a T-float x segment.
template <int T, class Sem>
struct RowBinTile {
    using W = typename TileWord<T>::type;
    using V = typename Sem::V;
    TileBits<T> bits;
    int tc;
    V xs[T];
    // colind and tile words stream through once per multiply: evict-first
    // loads keep L1 for the x segments that other tiles gather again
    __device__ __forceinline__ void load(const W* tiles, const int* colind, int j) {
        tc = __ldcs(colind + j);
        bits.load_stream(tiles, j);
    }
    __device__ __forceinline__ void load_x(const V* __restrict__ x, int ncols, cudaTextureObject_t xtex) {
        const long long base = (long long)tc * T;
        // T * sizeof(V) is a multiple of 16 for every T and word size
        constexpr int TEXELS = (int)(T * sizeof(V) / 16);
        if (base + T <= ncols) {
            if (xtex) {
                // texture pipe: a separate data path from the ld/st unit's
#pragma unroll
                for (int q = 0; q < TEXELS; ++q)
                    reinterpret_cast<uint4*>(xs)[q] = tex1Dfetch<uint4>(xtex, (int)(tc * TEXELS + q));
            } else {
                const uint4* p = reinterpret_cast<const uint4*>(x + base);
#pragma unroll
                for (int q = 0; q < TEXELS; ++q) reinterpret_cast<uint4*>(xs)[q] = __ldg(p + q);
            }
        } else {
#pragma unroll
            for (int c = 0; c < T; ++c) xs[c] = (base + c < ncols) ? __ldg(x + base + c) : Sem::zero();
        }
    }
    __device__ __forceinline__ void add_to(V (&acc)[T], const V*, int) const {
        if constexpr (T == 4 || !std::is_same<Sem, SemSumF32>::value) {
#pragma unroll
            for (int r = 0; r < T; ++r) {
                const uint32_t w = bits.row(r);
#pragma unroll
                for (int c = 0; c < T; ++c)
                    if (w & (1u << (T - 1 - c))) acc[r] = Sem::add(acc[r], xs[c]);
            }
        } else {
#pragma unroll
            for (int r = 0; r < T; ++r) {
                const uint32_t w = bits.row(r);
                float sum = 0.0f;
#pragma unroll
                for (int c = 0; c < T; ++c)
                    if (w & (1u << (T - 1 - c))) sum += xs[c];
                acc[r] += sum;
            }
        }
    }
};

// FP32 tile in sparse-column form (the default at T >= 16, an option below).
// load_x forms the column mask (OR of the rows) and loads x for its first K
// set columns, ascending; add_to adds them row by row, then walks any further
// columns one at a time.  Each row's sum runs over its set columns in
// ascending order with the dense form's association (per-tile sums at T >= 8,
// straight into acc at T = 4), so the two forms give bitwise-equal results.
template <int T>
struct SparseColTile {
    using W = typename TileWord<T>::type;
    static constexpr int K = SparseColsK<T>::value;
    TileBits<T> bits;
    int tc;
    uint32_t rest;      // set columns past the first K (bit T-1-c = column c)
    uint32_t cbit[K];   // column bit of gathered column k (0: none)
    float xv[K];
    const float* xrow;  // x + tc*T
    int lim;            // columns of this tile-column inside x
    __device__ __forceinline__ void load(const W* tiles, const int* colind, int j) {
        tc = __ldcs(colind + j);
        bits.load_stream(tiles, j);
    }
    __device__ __forceinline__ void load_x(const float* __restrict__ x, int ncols, cudaTextureObject_t) {
        uint32_t cm = 0;
#pragma unroll
        for (int r = 0; r < T; ++r) cm |= bits.row(r);
        const long long base = (long long)tc * T;
        xrow = x + base;
        lim = (int)(ncols - base < T ? ncols - base : T);
#pragma unroll
        for (int k = 0; k < K; ++k) {
            // the highest set bit is the lowest column
            const uint32_t b = cm ? (0x80000000u >> __clz(cm)) : 0u;
            const int c = T - 1 - (31 - __clz(b | 1u));
            cbit[k] = b;
            xv[k] = (b && c < lim) ? __ldg(xrow + c) : 0.0f;
            cm &= ~b;
        }
        rest = cm;
    }
    __device__ __forceinline__ void add_to(float (&acc)[T], const float*, int) const {
        if constexpr (T == 4) {
            // the dense T = 4 form adds each column straight into acc[r]
#pragma unroll
            for (int r = 0; r < T; ++r) {
                const uint32_t w = bits.row(r);
#pragma unroll
                for (int k = 0; k < K; ++k)
                    if (w & cbit[k]) acc[r] += xv[k];
            }
            for (uint32_t cm = rest; cm;) {
                const uint32_t b = 0x80000000u >> __clz(cm);
                const int c = T - 1 - (31 - __clz(b));
                const float xc = c < lim ? __ldg(xrow + c) : 0.0f;
#pragma unroll
                for (int r = 0; r < T; ++r)
                    if (bits.row(r) & b) acc[r] += xc;
                cm &= ~b;
            }
        } else {
            float sum[T];
#pragma unroll
            for (int r = 0; r < T; ++r) {
                const uint32_t w = bits.row(r);
                float s = 0.0f;
#pragma unroll
                for (int k = 0; k < K; ++k)
                    if (w & cbit[k]) s += xv[k];
                sum[r] = s;
            }
            for (uint32_t cm = rest; cm;) {
                const uint32_t b = 0x80000000u >> __clz(cm);
                const int c = T - 1 - (31 - __clz(b));
                const float xc = c < lim ? __ldg(xrow + c) : 0.0f;
#pragma unroll
                for (int r = 0; r < T; ++r)
                    if (bits.row(r) & b) sum[r] += xc;
                cm &= ~b;
            }
#pragma unroll
            for (int r = 0; r < T; ++r) acc[r] += sum[r];
        }
    }
};

// Register cap of the FP32 T = 8 dense and T = 32 set-column kernels and of
// the 64-frontier OR kernel at T = 4 (255: none; the FP32 T = 4 and 16 forms
// are capped through their launch bounds).  The 64-frontier cap: 36 warps per
// SM instead of 34 at 60 registers; R-MAT scale 18 with 64 frontiers 53.5
// instead of 61.4 us per call (48 spilled and took 58.9).
template <int T, class Sem, bool SPARSE> struct RowBinMaxReg {
    static constexpr bool f32 = std::is_same<Sem, SemSumF32>::value;
    static constexpr int value = (f32 && T == 8 && !SPARSE)                       ? 56
                                 : (f32 && T == 32 && SPARSE)                      ? 80
                                 : (T == 4 && std::is_same<Sem, SemOrU64>::value) ? 56
                                                                                   : 255;
};

template <int T, class Sem, bool SPARSE>
using LaneTile = typename std::conditional<(SPARSE && std::is_same<Sem, SemSumF32>::value), SparseColTile<T>,
                                           RowBinTile<T, Sem>>::type;

// Butterfly reduce-scatter of T values over a group of G lanes (group-local
// lane l), one shuffle step per lane bit S = G/2, G/4, ..., 1.  While a lane
// holds NV > 1 values a step halves them: the lane whose bit S is set keeps
// the upper half (and adds the partner's upper half to it), the other keeps
// the lower half.  Once one value is left the remaining steps add it across
// the lanes that share it.  `first` accumulates the index of the first row
// the lane holds; it ends with max(1, T/G) rows in acc[0..].  Every index is
// a compile-time constant, so acc stays in registers.
template <int T, class Sem, int NV, int S>
struct GroupReduce {
    using V = typename Sem::V;
    static __device__ __forceinline__ void run(V (&acc)[T], int l, int& first) {
        if constexpr (S >= 1) {
            if constexpr (NV > 1) {
                constexpr int H = NV / 2;
                const bool upper = (l & S) != 0;
#pragma unroll
                for (int k = 0; k < H; ++k) {
                    const V keep = upper ? acc[H + k] : acc[k];
                    const V give = upper ? acc[k] : acc[H + k];
                    acc[k] = Sem::add(keep, __shfl_xor_sync(FULL_MASK, give, S));
                }
                if (upper) first += H;
                GroupReduce<T, Sem, H, S / 2>::run(acc, l, first);
            } else {
                acc[0] = Sem::add(acc[0], __shfl_xor_sync(FULL_MASK, acc[0], S));
                GroupReduce<T, Sem, 1, S / 2>::run(acc, l, first);
            }
        }
    }
};

template <int T, class Sem, int G>
__device__ __forceinline__ int group_reduce(typename Sem::V (&acc)[T], int l) {
    int first = 0;
    GroupReduce<T, Sem, T, G / 2>::run(acc, l, first);
    return first;
}

template <int T, class Sem, int G, bool SPARSE>
__device__ __forceinline__ void rowbin_group(const RowBinArgs& a, int task, bool valid, int l) {
    using W = typename TileWord<T>::type;
    using V = typename Sem::V;
    constexpr int U = RowBinU<T>::value;
    const int4 t = valid ? __ldg(a.tasks + task) : make_int4(0, 0, 0, -2);
    const W* tiles = static_cast<const W*>(a.tiles);
    const V* x = static_cast<const V*>(a.x);
    LaneTile<T, Sem, SPARSE> tl[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int j = t.y + l + u * G;
        if (j < t.z) tl[u].load(tiles, a.colind, j);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int j = t.y + l + u * G;
        if (j < t.z) tl[u].load_x(x, a.ncols, a.xtex);
    }
    V acc[T];
#pragma unroll
    for (int r = 0; r < T; ++r) acc[r] = Sem::zero();
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int j = t.y + l + u * G;
        if (j < t.z) tl[u].add_to(acc, x, a.ncols);
    }
    const int first = group_reduce<T, Sem, G>(acc, l);
    constexpr int NV = T >= G ? T / G : 1;
    // with T < G, G/T lanes share each row: the lowest one writes it
    const bool writer = (T >= G) || ((l & (G / T - 1)) == 0);
    if (!valid || !writer || t.w == -2) return;
    const size_t off = (size_t)(t.w < 0 ? t.x : t.w) * T + first;
    V* dst = static_cast<V*>(t.w < 0 ? a.y : a.partials) + off;
    if (t.w < 0 && a.mask) {
        const V* mk = static_cast<const V*>(a.mask) + off;
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = Sem::clear(acc[k], mk[k]);
    }
    const bool acc_old = t.w < 0 && a.accumulate;
    if constexpr ((NV * sizeof(V)) % 16 == 0) {
        constexpr int PER = 16 / sizeof(V);
#pragma unroll
        for (int q = 0; q < NV / PER; ++q) {
            uint4* p = reinterpret_cast<uint4*>(dst) + q;
            V o[PER];
#pragma unroll
            for (int e = 0; e < PER; ++e) o[e] = acc[q * PER + e];
            if (acc_old) {
                const uint4 old = *p;
                const V* ov = reinterpret_cast<const V*>(&old);
#pragma unroll
                for (int e = 0; e < PER; ++e) o[e] = Sem::add(ov[e], o[e]);
            }
            *p = *reinterpret_cast<const uint4*>(o);
        }
    } else {
#pragma unroll
        for (int k = 0; k < NV; ++k) dst[k] = acc_old ? Sem::add(dst[k], acc[k]) : acc[k];
    }
}

template <int T, class Sem, bool SPARSE>
// T = 4 with 32-bit values fits 32 registers, so 64 warps fit on an SM (90 us
// instead of 102 us for R-MAT scale 20).  Register caps that buy occupancy
// for a few bytes of spills, R-MAT scale 20: the FP32 T = 8 form at 56 (36
// warps per SM instead of 32 at 63; 139 instead of 143 us, while 48 was
// slower), the T = 16 set-column form at 64 (32 warps instead of 28 at 72;
// 264 instead of 278 us) and the T = 32 set-column form at 80 (24 warps
// instead of 20 at 86; 645 instead of 690 us; 72 spilled 356 bytes and was
// slower).  Launched as two-warp blocks: 87 us instead of 90 us with 8-warp
// blocks at T = 4, 143 us instead of 155 us at T = 8.
__global__ void __launch_bounds__(256, (T == 4 && sizeof(typename Sem::V) == 4) ? (SPARSE ? 5 : 8)
                                       : (T == 16 && SPARSE)                    ? 4
                                                                                : 1)
    __maxnreg__((RowBinMaxReg<T, Sem, SPARSE>::value)) rowbin_spmv_kernel(RowBinArgs a) {
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (warp >= a.warp_off[RB_BINS]) return;
    // bin of this warp; the offsets are read with constant indices only (a
    // runtime index into the parameter arrays would copy them to local memory)
    int k = 0, woff = a.warp_off[0], toff = a.task_off[0], tend = a.task_off[1];
#pragma unroll
    for (int kk = 1; kk < RB_BINS; ++kk) {
        if (warp >= a.warp_off[kk]) {
            k = kk;
            woff = a.warp_off[kk];
            toff = a.task_off[kk];
            tend = a.task_off[kk + 1];
        }
    }
    const int b = RB_BINS - 1 - k;  // plan slot k holds bin RB_BINS-1-k
    const int per_warp = 32 >> b;  // tasks per warp in bin b (G = 1 << b)
    const int task = toff + (warp - woff) * per_warp + (lane >> b);
    const bool valid = task < tend;
    const int l = lane & ((1 << b) - 1);
    switch (b) {
        case 0: rowbin_group<T, Sem, 1, SPARSE>(a, task, valid, l); break;
        case 1: rowbin_group<T, Sem, 2, SPARSE>(a, task, valid, l); break;
        case 2: rowbin_group<T, Sem, 4, SPARSE>(a, task, valid, l); break;
        case 3: rowbin_group<T, Sem, 8, SPARSE>(a, task, valid, l); break;
        case 4: rowbin_group<T, Sem, 16, SPARSE>(a, task, valid, l); break;
        default: rowbin_group<T, Sem, 32, SPARSE>(a, task, valid, l); break;
    }
}

// Long rows: y[row] (+)= the combination of its segment partials (AND NOT
// mask for masked OR products).  long_rows[i] = (row, first slot, slot
// count); the plan lists the rows with at most FIX_G slots first.  Those get
// FIX_G lanes each (32 / FIX_G rows per warp, one slot per lane); the others a
// warp each, lane k folding slots k, k + 32, ... in order.  A group then
// combines its lane partials with the main kernel's butterfly, so the order is
// fixed for each row.
constexpr int FIX_G = 8;

__host__ __device__ __forceinline__ int fixup_warps(int nlong, int nshort) {
    return (nshort + 32 / FIX_G - 1) / (32 / FIX_G) + (nlong - nshort);
}

template <int T, class Sem, int G>
__device__ __forceinline__ void fixup_group(const int4* __restrict__ long_rows, int idx, bool valid, int l,
                                            const typename Sem::V* __restrict__ partials, typename Sem::V* y,
                                            const typename Sem::V* __restrict__ mask, int accumulate) {
    using V = typename Sem::V;
    const int4 L = valid ? __ldg(long_rows + idx) : make_int4(0, 0, 0, 0);
    V acc[T];
#pragma unroll
    for (int r = 0; r < T; ++r) acc[r] = Sem::zero();
    // up to four slots' loads in flight per step (slots of at most 32 bytes),
    // added in slot order
    constexpr int UNR = T * sizeof(V) <= 32 ? 4 : 1;
    for (int k0 = l; k0 < L.z; k0 += UNR * G) {
        V v[UNR][T];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const int k = k0 + G * u;
            if (k < L.z) {
                const uint4* p = reinterpret_cast<const uint4*>(partials + (size_t)(L.y + k) * T);
#pragma unroll
                for (int q = 0; q < (int)(T * sizeof(V) / 16); ++q) reinterpret_cast<uint4*>(v[u])[q] = __ldg(p + q);
            }
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u)
            if (k0 + G * u < L.z) {
#pragma unroll
                for (int r = 0; r < T; ++r) acc[r] = Sem::add(acc[r], v[u][r]);
            }
    }
    const int first = group_reduce<T, Sem, G>(acc, l);
    constexpr int NV = T >= G ? T / G : 1;
    if (!valid || !(T >= G || (l & (G / T - 1)) == 0)) return;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const size_t o = (size_t)L.x * T + first + k;
        V s = acc[k];
        if (mask) s = Sem::clear(s, mask[o]);
        y[o] = accumulate ? Sem::add(y[o], s) : s;
    }
}

template <int T, class Sem>
__global__ void __launch_bounds__(256)
rowbin_fixup_kernel(const int4* __restrict__ long_rows, int nlong, int nshort,
                    const typename Sem::V* __restrict__ partials, typename Sem::V* __restrict__ y,
                    const typename Sem::V* __restrict__ mask, int accumulate) {
    griddep_wait();  // launched behind the main kernel: its partials
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    const int short_warps = (nshort + 32 / FIX_G - 1) / (32 / FIX_G);
    if (w < short_warps) {  // warp-uniform branch
        const int idx = w * (32 / FIX_G) + lane / FIX_G;
        fixup_group<T, Sem, FIX_G>(long_rows, idx, idx < nshort, lane & (FIX_G - 1), partials, y, mask,
                                   accumulate);
        return;
    }
    const int lr = nshort + (w - short_warps);
    if (lr >= nlong) return;  // warp-uniform
    fixup_group<T, Sem, 32>(long_rows, lr, true, lane, partials, y, mask, accumulate);
}

// ---- plan -----------------------------------------------------------------------------
struct RowBinPlanHost {
    std::vector<int4> tasks;
    std::vector<int4> long_rows;
    int nlong_short = 0;
    int task_off[RB_BINS + 1];
    int warp_off[RB_BINS + 1];
    int nslots = 0;
};

static RowBinPlanHost build_rowbin_plan(const std::vector<int>& rowptr, int T, int UL) {
    const int U = T <= 8 ? 4 : T == 16 ? 2 : 1;
    const int nb = (int)rowptr.size() - 1;
    const int seg = 32 * UL;
    std::vector<std::vector<int4>> bins(RB_BINS);
    RowBinPlanHost p;
    for (int i = 0; i < nb; ++i) {
        const int b0 = rowptr[i], m = rowptr[i + 1] - b0;
        int b = 0;
        while (b < RB_BINS - 1 && m > (U << b)) ++b;
        if (m <= seg) {
            bins[b].push_back(make_int4(i, b0, b0 + m, -1));
        } else {
            const int nseg = (m + seg - 1) / seg;
            p.long_rows.push_back(make_int4(i, p.nslots, nseg, 0));
            for (int s = 0; s < nseg; ++s)
                bins[RB_BINS - 1].push_back(make_int4(i, b0 + s * seg, std::min(b0 + (s + 1) * seg, b0 + m),
                                                      p.nslots + s));
            p.nslots += nseg;
        }
    }
    // long rows with at most FIX_G slots first (the fix-up's narrow groups)
    std::stable_partition(p.long_rows.begin(), p.long_rows.end(), [](const int4& L) { return L.z <= FIX_G; });
    p.nlong_short = (int)std::count_if(p.long_rows.begin(), p.long_rows.end(),
                                       [](const int4& L) { return L.z <= FIX_G; });
    // plan slot k holds bin RB_BINS-1-k: the long-row warps come first, so
    // they start early and the short bins fill the tail
    p.task_off[0] = 0;
    p.warp_off[0] = 0;
    for (int k = 0; k < RB_BINS; ++k) {
        const int b = RB_BINS - 1 - k;
        p.tasks.insert(p.tasks.end(), bins[b].begin(), bins[b].end());
        p.task_off[k + 1] = (int)p.tasks.size();
        const int per_warp = 32 >> b;
        p.warp_off[k + 1] = p.warp_off[k] + ((int)bins[b].size() + per_warp - 1) / per_warp;
    }
    return p;
}

b2sr_status rowbin_plan_create(const int* d_rowptr, int nb, int T, bool bits, RowBinPlan* out, cudaStream_t s) {
    std::vector<int> rp((size_t)nb + 1);
    cudaError_t e = cudaMemcpyAsync(rp.data(), d_rowptr, sizeof(int) * rp.size(), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return B2SR_ERR_CUDA;
    }
    RowBinPlanHost h = build_rowbin_plan(rp, T, bits ? rb_long_u(T) : (T <= 8 ? 4 : T == 16 ? 2 : 1));
    RowBinPlan p;
    p.ntasks = (int)h.tasks.size();
    p.nlong = (int)h.long_rows.size();
    p.nlong_short = h.nlong_short;
    p.nslots = h.nslots;
    for (int b = 0; b <= RB_BINS; ++b) {
        p.task_off[b] = h.task_off[b];
        p.warp_off[b] = h.warp_off[b];
    }
    p.d_tasks = static_cast<int4*>(dev_alloc(sizeof(int4) * (size_t)std::max(p.ntasks, 1)));
    p.d_long = static_cast<int4*>(dev_alloc(sizeof(int4) * (size_t)std::max(p.nlong, 1)));
    if (!p.d_tasks || !p.d_long) {
        dev_free(p.d_tasks);
        dev_free(p.d_long);
        return B2SR_ERR_ALLOC;
    }
    e = cudaSuccess;
    if (p.ntasks) e = cudaMemcpy(p.d_tasks, h.tasks.data(), sizeof(int4) * (size_t)p.ntasks, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && p.nlong)
        e = cudaMemcpy(p.d_long, h.long_rows.data(), sizeof(int4) * (size_t)p.nlong, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        dev_free(p.d_tasks);
        dev_free(p.d_long);
        return B2SR_ERR_CUDA;
    }
    *out = p;
    return B2SR_SUCCESS;
}

void rowbin_plan_free(RowBinPlan* p) {
    dev_free(p->d_tasks);
    dev_free(p->d_long);
    p->d_tasks = nullptr;
    p->d_long = nullptr;
}

size_t rowbin_scratch_bytes(const RowBinPlan& p, int T, int value_bytes) {
    return (size_t)value_bytes * (size_t)std::max(p.nslots, 1) * T;
}

template <int T, class Sem>
static b2sr_status run_rowbin(const RowBinPlan& p, const MatView& A, const void* x, void* y, const void* mask,
                              int accumulate, void* partials, cudaTextureObject_t xtex, bool sparse, cudaStream_t s) {
    using V = typename Sem::V;
    RowBinArgs a;
    a.colind = A.colind;
    a.tiles = A.tiles;
    a.x = x;
    a.y = y;
    a.mask = mask;
    a.tasks = p.d_tasks;
    a.partials = partials;
    for (int b = 0; b <= RB_BINS; ++b) {
        a.task_off[b] = p.task_off[b];
        a.warp_off[b] = p.warp_off[b];
    }
    a.ncols = A.ncols;
    a.accumulate = accumulate;
    a.xtex = xtex;
    const int warps = p.warp_off[RB_BINS];
    int launches = 0;
    if (warps > 0) {
        kernel_timer_mark(s, true);
        // two-warp blocks: finer scheduling
        if constexpr (std::is_same<Sem, SemSumF32>::value) {
            if (sparse) rowbin_spmv_kernel<T, Sem, true><<<(warps + 1) / 2, 64, 0, s>>>(a);
            else rowbin_spmv_kernel<T, Sem, false><<<(warps + 1) / 2, 64, 0, s>>>(a);
        } else {
            rowbin_spmv_kernel<T, Sem, false><<<(warps + 1) / 2, 64, 0, s>>>(a);
        }
        kernel_timer_mark(s, false);
        B2SR_LAUNCH_CHECK();
        ++launches;
    }
    if (p.nlong > 0) {
        B2SR_CUDA_TRY(launch_dependent(rowbin_fixup_kernel<T, Sem>, (unsigned)((fixup_warps(p.nlong, p.nlong_short) + 7) / 8),
                                       256u, s, (const int4*)p.d_long, p.nlong, p.nlong_short,
                                       static_cast<const V*>(partials), static_cast<V*>(y),
                                       static_cast<const V*>(mask), accumulate));
        ++launches;
    }
    add_launch_count(launches);
    return B2SR_SUCCESS;
}

template <class Sem>
static b2sr_status rowbin_dispatch(const RowBinPlan& p, const MatView& A, const void* x, void* y, const void* mask,
                                   int accumulate, void* scratch, cudaTextureObject_t xtex, bool sparse,
                                   cudaStream_t s) {
    switch (A.T) {
        case 4: return run_rowbin<4, Sem>(p, A, x, y, mask, accumulate, scratch, xtex, sparse, s);
        case 8: return run_rowbin<8, Sem>(p, A, x, y, mask, accumulate, scratch, xtex, sparse, s);
        case 16: return run_rowbin<16, Sem>(p, A, x, y, mask, accumulate, scratch, xtex, sparse, s);
        case 32: return run_rowbin<32, Sem>(p, A, x, y, mask, accumulate, scratch, xtex, sparse, s);
    }
    return B2SR_ERR_INVALID_VALUE;
}

b2sr_status rowbin_spmv(const RowBinPlan& p, const MatView& A, const float* x, float* y, int accumulate,
                        void* scratch, cudaTextureObject_t xtex, bool sparse_cols, cudaStream_t s) {
    return rowbin_dispatch<SemSumF32>(p, A, x, y, nullptr, accumulate, scratch, xtex, sparse_cols, s);
}

b2sr_status rowbin_multi_bits(const RowBinPlan& p, const MatView& A, const void* x, void* y, const void* mask,
                              int word_bits, int accumulate, void* scratch, cudaTextureObject_t xtex,
                              cudaStream_t s) {
    if (word_bits == 32) return rowbin_dispatch<SemOrU32>(p, A, x, y, mask, accumulate, scratch, xtex, false, s);
    if (word_bits == 64) return rowbin_dispatch<SemOrU64>(p, A, x, y, mask, accumulate, scratch, xtex, false, s);
    return B2SR_ERR_INVALID_VALUE;
}

// ---- bit-vector variants on the row-binned plan ------------------------------------------
// The same plan and lane groups, with one x word (T bits) per tile-column:
//   KIND 0  bin_bin_bin:  bit r of the tile-row's word = OR over its tiles of
//                         (row r AND x word) != 0      (bsrbmv.cu:277-613)
//   KIND 1  the same AND NOT a mask word (masked BFS step, bsrbmv.cu:1083-1229)
//   KIND 2  bin_bin_count: y[r] = sum of popc(row r AND x word), int32
//   KIND 3  bin_bin_full:  the same counts as FP32      (bsrbmv.cu:618-821)
// Counts are integers, so their sums are exact in any order; the OR is too.
struct RowBinBitsArgs {
    const int* colind;
    const void* tiles;
    const void* x;
    void* y;
    const void* mask;
    const int4* tasks;
    void* partials;  // long-row segment slots: one word (KIND 0/1) or T ints (KIND 2/3)
    int task_off[RB_BINS + 1];
    int warp_off[RB_BINS + 1];
    int accumulate;
    const int* push_ctl;  // auto direction: the push kernel's counters (null: always pull)
    int push_pct;
    long long nt;
};

// In auto direction the pull kernels return when the push kernel took the product.
__device__ __forceinline__ bool pull_skipped(const RowBinBitsArgs& a) {
    return a.push_ctl != nullptr && push_chosen(a.push_ctl, 1, a.nt, a.push_pct);
}

struct SemSumI32 {
    using V = int;
    static __device__ __forceinline__ V zero() { return 0; }
    static __device__ __forceinline__ V add(V a, V b) { return a + b; }
    static __device__ __forceinline__ V clear(V a, V) { return a; }
};

template <int T, int KIND, int G>
__device__ __forceinline__ void bits_group(const RowBinBitsArgs& a, int task, bool valid, int l) {
    using W = typename TileWord<T>::type;
    constexpr int U = RowBinTaskU<T, G>::value;
    const int4 t = valid ? __ldg(a.tasks + task) : make_int4(0, 0, 0, -2);
    const W* tiles = static_cast<const W*>(a.tiles);
    const W* x = static_cast<const W*>(a.x);
    int tc[U];
    TileBits<T> bits[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int j = t.y + l + u * G;
        tc[u] = -1;
        if (j < t.z) {
            tc[u] = __ldcs(a.colind + j);
            bits[u].load_stream(tiles, j);
        }
    }
    uint32_t xw[U];
#pragma unroll
    for (int u = 0; u < U; ++u) xw[u] = tc[u] >= 0 ? (uint32_t)__ldg(x + tc[u]) : 0u;
    if constexpr (KIND <= 1) {
        uint32_t m = 0;
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (tc[u] >= 0) {
#pragma unroll
                for (int r = 0; r < T; ++r) m |= ((bits[u].row(r) & xw[u]) != 0u ? 1u : 0u) << (T - 1 - r);
            }
#pragma unroll
        for (int sh = G / 2; sh >= 1; sh >>= 1) m |= __shfl_xor_sync(FULL_MASK, m, sh);
        if (!valid || l != 0 || t.w == -2) return;
        if (t.w >= 0) {
            static_cast<uint32_t*>(a.partials)[t.w] = m;
            return;
        }
        W* y = static_cast<W*>(a.y) + t.x;
        if (KIND == 1) m &= ~(uint32_t)__ldg(static_cast<const W*>(a.mask) + t.x);
        *y = (W)(a.accumulate ? ((uint32_t)*y | m) : m);
    } else {
        int acc[T];
#pragma unroll
        for (int r = 0; r < T; ++r) acc[r] = 0;
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (tc[u] >= 0) {
#pragma unroll
                for (int r = 0; r < T; ++r) acc[r] += __popc(bits[u].row(r) & xw[u]);
            }
        const int first = group_reduce<T, SemSumI32, G>(acc, l);
        constexpr int NV = T >= G ? T / G : 1;
        const bool writer = (T >= G) || ((l & (G / T - 1)) == 0);
        if (!valid || !writer || t.w == -2) return;
        if (t.w >= 0) {
            int* dst = static_cast<int*>(a.partials) + (size_t)t.w * T + first;
#pragma unroll
            for (int k = 0; k < NV; ++k) dst[k] = acc[k];
            return;
        }
        const size_t off = (size_t)t.x * T + first;
        if constexpr (KIND == 2) {
            int* dst = static_cast<int*>(a.y) + off;
#pragma unroll
            for (int k = 0; k < NV; ++k) dst[k] = a.accumulate ? dst[k] + acc[k] : acc[k];
        } else {
            float* dst = static_cast<float*>(a.y) + off;
#pragma unroll
            for (int k = 0; k < NV; ++k) dst[k] = a.accumulate ? dst[k] + (float)acc[k] : (float)acc[k];
        }
    }
}

// T <= 8 fits 32 registers: 64 warps per SM.  So do the T = 16 bit kernels
// (bin_bin_bin, masked) without spills: 64 warps per SM instead of 48 at 40,
// R-MAT scale 20 121.5 instead of 133.1 us per call (the count kinds and
// T = 32 spill at such caps).
template <int T, int KIND>
__global__ void __launch_bounds__(256, T <= 8 ? 8 : 1) __maxnreg__((T == 16 && KIND <= 1 ? 32 : 255))
    rowbin_bits_kernel(RowBinBitsArgs a) {
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (warp >= a.warp_off[RB_BINS] || pull_skipped(a)) return;
    int k = 0, woff = a.warp_off[0], toff = a.task_off[0], tend = a.task_off[1];
#pragma unroll
    for (int kk = 1; kk < RB_BINS; ++kk) {
        if (warp >= a.warp_off[kk]) {
            k = kk;
            woff = a.warp_off[kk];
            toff = a.task_off[kk];
            tend = a.task_off[kk + 1];
        }
    }
    const int b = RB_BINS - 1 - k;  // plan slot k holds bin RB_BINS-1-k
    const int per_warp = 32 >> b;
    const int task = toff + (warp - woff) * per_warp + (lane >> b);
    const bool valid = task < tend;
    const int l = lane & ((1 << b) - 1);
    switch (b) {
        case 0: bits_group<T, KIND, 1>(a, task, valid, l); break;
        case 1: bits_group<T, KIND, 2>(a, task, valid, l); break;
        case 2: bits_group<T, KIND, 4>(a, task, valid, l); break;
        case 3: bits_group<T, KIND, 8>(a, task, valid, l); break;
        case 4: bits_group<T, KIND, 16>(a, task, valid, l); break;
        default: bits_group<T, KIND, 32>(a, task, valid, l); break;
    }
}

// Long rows: combine the segment slots (OR of words, or exact int sums), with
// the lane groups of rowbin_fixup_kernel.
template <int T, int KIND, int G>
__device__ __forceinline__ void bits_fixup_group(const RowBinBitsArgs& a, const int4* __restrict__ long_rows, int idx,
                                                 bool valid, int l) {
    using W = typename TileWord<T>::type;
    const int4 L = valid ? __ldg(long_rows + idx) : make_int4(0, 0, 0, 0);
    if constexpr (KIND <= 1) {
        uint32_t m = 0;
        for (int k = l; k < L.z; k += G) m |= __ldg(static_cast<const uint32_t*>(a.partials) + L.y + k);
#pragma unroll
        for (int sh = G / 2; sh >= 1; sh >>= 1) m |= __shfl_xor_sync(FULL_MASK, m, sh);
        if (!valid || l != 0) return;
        W* y = static_cast<W*>(a.y) + L.x;
        if (KIND == 1) m &= ~(uint32_t)__ldg(static_cast<const W*>(a.mask) + L.x);
        *y = (W)(a.accumulate ? ((uint32_t)*y | m) : m);
    } else {
        const int* part = static_cast<const int*>(a.partials);
        int acc[T];
#pragma unroll
        for (int r = 0; r < T; ++r) acc[r] = 0;
        for (int k = l; k < L.z; k += G) {
            const int4* p = reinterpret_cast<const int4*>(part + (size_t)(L.y + k) * T);
#pragma unroll
            for (int q = 0; q < T / 4; ++q) {
                const int4 v = __ldg(p + q);
                acc[4 * q] += v.x;
                acc[4 * q + 1] += v.y;
                acc[4 * q + 2] += v.z;
                acc[4 * q + 3] += v.w;
            }
        }
        const int first = group_reduce<T, SemSumI32, G>(acc, l);
        constexpr int NV = T >= G ? T / G : 1;
        if (!valid || !(T >= G || (l & (G / T - 1)) == 0)) return;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const size_t o = (size_t)L.x * T + first + k;
            if constexpr (KIND == 2) {
                int* y = static_cast<int*>(a.y);
                y[o] = a.accumulate ? y[o] + acc[k] : acc[k];
            } else {
                float* y = static_cast<float*>(a.y);
                y[o] = a.accumulate ? y[o] + (float)acc[k] : (float)acc[k];
            }
        }
    }
}

template <int T, int KIND>
__global__ void __launch_bounds__(256) rowbin_bits_fixup_kernel(RowBinBitsArgs a, const int4* __restrict__ long_rows,
                                                                int nlong, int nshort) {
    griddep_wait();  // launched behind the main kernel: its partials
    if (pull_skipped(a)) return;
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    const int short_warps = (nshort + 32 / FIX_G - 1) / (32 / FIX_G);
    if (w < short_warps) {  // warp-uniform branch
        const int idx = w * (32 / FIX_G) + lane / FIX_G;
        bits_fixup_group<T, KIND, FIX_G>(a, long_rows, idx, idx < nshort, lane & (FIX_G - 1));
        return;
    }
    const int lr = nshort + (w - short_warps);
    if (lr >= nlong) return;  // warp-uniform
    bits_fixup_group<T, KIND, 32>(a, long_rows, lr, true, lane);
}

// Auto direction with a push hint: one thread reads the classify pass's
// decision and, only when the push did not take the product (the hint was
// wrong), launches the pull kernel and its fix-up from the device (tail
// launches: they start when this grid ends, in launch order, and the host
// stream's next work waits for them).  A tail launch costs 15-20 us more
// than a host launch, which the hint keeps to the calls where the frontier
// crosses the threshold.
template <int T, int KIND>
__global__ void rowbin_bits_gate_kernel(RowBinBitsArgs a, unsigned blocks, unsigned threads, const int4* long_rows,
                                        int nlong, int nshort, unsigned fix_blocks) {
    // launched behind the push kernel: wait for all of it (so the work after
    // this grid, which waits for this grid and its tail launches, follows it)
    griddep_wait();
    if (threadIdx.x != 0 || blockIdx.x != 0 || pull_skipped(a)) return;
    a.push_ctl = nullptr;  // the pull runs unconditionally from here
    if (blocks > 0) rowbin_bits_kernel<T, KIND><<<blocks, threads, 0, cudaStreamTailLaunch>>>(a);
    if (nlong > 0)
        rowbin_bits_fixup_kernel<T, KIND><<<fix_blocks, 256, 0, cudaStreamTailLaunch>>>(a, long_rows, nlong, nshort);
}

size_t rowbin_bits_scratch_bytes(const RowBinPlan& p, int T) {
    return (size_t)std::max(p.nslots, 1) * T * sizeof(int);
}

template <int T, int KIND>
static b2sr_status run_rowbin_bits(const RowBinPlan& p, const MatView& A, const void* x, void* y, const void* mask,
                                   int accumulate, void* partials, const PushLink& link, bool timed,
                                   cudaStream_t s) {
    RowBinBitsArgs a;
    a.colind = A.colind;
    a.tiles = A.tiles;
    a.x = x;
    a.y = y;
    a.mask = mask;
    a.tasks = p.d_tasks;
    a.partials = partials;
    for (int b = 0; b <= RB_BINS; ++b) {
        a.task_off[b] = p.task_off[b];
        a.warp_off[b] = p.warp_off[b];
    }
    a.accumulate = accumulate;
    a.push_ctl = link.ctl;
    a.push_pct = link.pct;
    a.nt = link.nt;
    const int warps = p.warp_off[RB_BINS];
    int launches = 0;
    const unsigned fix_blocks = (unsigned)((fixup_warps(p.nlong, p.nlong_short) + 7) / 8);
    if (link.ctl && link.gate) {
        // the pull is launched from the device only when it is chosen
        const int wpb = T <= 8 ? 2 : 8;
        B2SR_CUDA_TRY(launch_dependent(rowbin_bits_gate_kernel<T, KIND>, 1u, 32u, s, a,
                                       (unsigned)((warps + wpb - 1) / wpb), 32u * wpb, (const int4*)p.d_long,
                                       p.nlong, p.nlong_short, fix_blocks));
        add_launch_count(1);
        return B2SR_SUCCESS;
    }
    if (warps > 0) {
        // two-warp blocks at T <= 8 (finer scheduling: faster than 256-thread
        // blocks), but eight-warp blocks behind an auto-direction push, where
        // most blocks only retire
        const int wpb = (T <= 8 && !link.ctl) ? 2 : 8;
        if (timed) kernel_timer_mark(s, true);
        rowbin_bits_kernel<T, KIND><<<(warps + wpb - 1) / wpb, 32 * wpb, 0, s>>>(a);
        if (timed) kernel_timer_mark(s, false);
        B2SR_LAUNCH_CHECK();
        ++launches;
    }
    if (p.nlong > 0) {
        B2SR_CUDA_TRY(launch_dependent(rowbin_bits_fixup_kernel<T, KIND>, fix_blocks, 256u, s, a,
                                       (const int4*)p.d_long, p.nlong, p.nlong_short));
        ++launches;
    }
    add_launch_count(launches);
    return B2SR_SUCCESS;
}

template <int T>
static b2sr_status bits_kind(int kind, const RowBinPlan& p, const MatView& A, const void* x, void* y,
                             const void* mask, int accumulate, void* partials, const PushLink& link, bool timed,
                             cudaStream_t s) {
    switch (kind) {
        case 0: return run_rowbin_bits<T, 0>(p, A, x, y, mask, accumulate, partials, link, timed, s);
        case 1: return run_rowbin_bits<T, 1>(p, A, x, y, mask, accumulate, partials, link, timed, s);
        case 2: return run_rowbin_bits<T, 2>(p, A, x, y, mask, accumulate, partials, link, timed, s);
        case 3: return run_rowbin_bits<T, 3>(p, A, x, y, mask, accumulate, partials, link, timed, s);
    }
    return B2SR_ERR_INVALID_VALUE;
}

b2sr_status rowbin_bits(const RowBinPlan& p, const MatView& A, int kind, const void* x, void* y, const void* mask,
                        int accumulate, void* partials, const PushLink& link, bool timed, cudaStream_t s) {
    switch (A.T) {
        case 4: return bits_kind<4>(kind, p, A, x, y, mask, accumulate, partials, link, timed, s);
        case 8: return bits_kind<8>(kind, p, A, x, y, mask, accumulate, partials, link, timed, s);
        case 16: return bits_kind<16>(kind, p, A, x, y, mask, accumulate, partials, link, timed, s);
        case 32: return bits_kind<32>(kind, p, A, x, y, mask, accumulate, partials, link, timed, s);
    }
    return B2SR_ERR_INVALID_VALUE;
}

// ---- texture objects over dense vectors --------------------------------------------------
// A cache of linear uint4 texture objects keyed by (pointer, bytes, device):
// repeated multiplies with the same x buffer reuse one object.  Objects are
// never destroyed while the library is loaded, because a kernel still in
// flight or a captured CUDA graph may hold the handle; once the cache is full,
// new vectors get no texture (0) and the kernels gather through ld.global.
namespace {
using TexKey = std::tuple<const void*, size_t, int>;  // (pointer, bytes, device)
std::mutex g_tex_mu;
std::map<TexKey, cudaTextureObject_t> g_tex;
constexpr size_t TEX_CACHE = 4096;
}  // namespace

cudaTextureObject_t vector_texture(const void* ptr, size_t bytes) {
    bytes = bytes / 16 * 16;
    if (!ptr || bytes == 0) return 0;
    int dev = 0;
    cudaGetDevice(&dev);
    int align = 0;
    if (cudaDeviceGetAttribute(&align, cudaDevAttrTextureAlignment, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (align > 0 && (uintptr_t)ptr % (uintptr_t)align != 0) return 0;
    if (bytes / 16 > (size_t)(1u << 27)) return 0;  // linear 1D texture width limit
    std::lock_guard<std::mutex> lk(g_tex_mu);
    const TexKey key(ptr, bytes, dev);
    auto it = g_tex.find(key);
    if (it != g_tex.end()) return it->second;
    if (g_tex.size() >= TEX_CACHE) return 0;
    cudaResourceDesc rd = {};
    rd.resType = cudaResourceTypeLinear;
    rd.res.linear.devPtr = const_cast<void*>(ptr);
    rd.res.linear.desc = cudaCreateChannelDesc<uint4>();
    rd.res.linear.sizeInBytes = bytes;
    cudaTextureDesc td = {};
    td.readMode = cudaReadModeElementType;
    cudaTextureObject_t t = 0;
    if (cudaCreateTextureObject(&t, &rd, &td, nullptr) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    g_tex.emplace(key, t);
    return t;
}

}  // namespace b2sr
