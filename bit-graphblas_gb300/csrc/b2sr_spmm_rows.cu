// Row-task B2SR x dense multiply: Y = A . X with X [ncols, k] and Y [nb*T, k]
// row-major, FP32 or FP64 (bin_full_full on feature blocks; the adjoint
// dX = A^T . dY is the same kernel on the transposed B2SR).  A task covers a
// whole tile-row at T = 4 and 8, and one group of 8 of its rows at T = 16
// and 32.
//
// Plan (host, once per matrix): one task per tile-row; a tile-row longer
// than spmm_rows_seg() tiles (a share of one resident warp's part of all the
// tiles) is cut into near-equal segments whose partial rows go to slots.  The warp that finishes a row's last segment (a per-row
// arrival counter) adds the row's slots in segment order and writes Y, so a
// multiply is one launch.  Warps take (column block, task) work items from a
// device queue (an atomic counter); long tasks are handed out first, so the
// queue ends on short ones (R-MAT hubs sit all over the vertex range, and in
// row order the last items could be the longest).  The queue and
// arrival counters live in a zeroed per-(matrix, stream) state buffer that
// the kernel's last warp leaves zeroed again, so no launch needs a memset.
//
// Inside a task a warp walks its tiles 32 at a time, one tile per lane.  The
// lanes' set bits are appended to T item lists in shared memory, one per
// tile row r, in tile then column order: the positions come from one warp
// scan of the per-row bit counts (packed several rows to a word).  The lists
// grow over many 32-tile steps (an R-MAT step holds ~8 items per row) and are
// consumed only when one would overflow or the task ends, so a row's items
// come in long runs.  The warp walks each list eight items per lane at a time,
// every lane loading its VEC columns of the eight X rows before adding them
// into acc[r] (a compile-time index), so eight coalesced row loads per lane
// are in flight; the rest of a list goes four (predicated) at a time.  The
// summation order is fixed, so the result does not depend on scheduling.
#include <algorithm>
#include <type_traits>
#include <vector>

#include "b2sr_spmv_impl.cuh"

namespace b2sr {

namespace {

constexpr int ROWS_CAP = 256;    // item capacity of each tile row's region (ints); a step adds <= 32*T
constexpr int ROWS_WARPS = 8;    // warps per block
constexpr int ROWS_BATCH = 8;    // X-row loads in flight per lane

template <typename V, int VEC> struct RowsVec;
template <> struct RowsVec<float, 1> { using type = float; };
template <> struct RowsVec<float, 2> { using type = float2; };
template <> struct RowsVec<float, 4> { using type = float4; };
template <> struct RowsVec<double, 1> { using type = double; };
template <> struct RowsVec<double, 2> { using type = double2; };

template <typename V, int VEC>
__device__ __forceinline__ void rows_load(V (&out)[VEC], const V* p, bool full, int nvalid) {
    if (full) {
        using VT = typename RowsVec<V, VEC>::type;
        const VT v = __ldg(reinterpret_cast<const VT*>(p));
        const V* e = reinterpret_cast<const V*>(&v);
#pragma unroll
        for (int i = 0; i < VEC; ++i) out[i] = e[i];
    } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i) out[i] = i < nvalid ? __ldg(p + i) : V(0);
    }
}

// acc += v element-wise; FP32 pairs as one packed two-lane add (add.rn.f32x2:
// two IEEE round-to-nearest adds, bitwise the same as the scalar ones).
template <typename V, int VEC>
__device__ __forceinline__ void rows_add(V (&acc)[VEC], const V (&v)[VEC]) {
    if constexpr (std::is_same<V, float>::value && VEC % 2 == 0) {
#pragma unroll
        for (int i = 0; i < VEC; i += 2) {
            unsigned long long x, y;
            asm("mov.b64 %0, {%1, %2};" : "=l"(x) : "f"(acc[i]), "f"(acc[i + 1]));
            asm("mov.b64 %0, {%1, %2};" : "=l"(y) : "f"(v[i]), "f"(v[i + 1]));
            asm("add.rn.f32x2 %0, %0, %1;" : "+l"(x) : "l"(y));
            asm("mov.b64 {%0, %1}, %2;" : "=f"(acc[i]), "=f"(acc[i + 1]) : "l"(x));
        }
        return;
    }
#pragma unroll
    for (int e = 0; e < VEC; ++e) acc[e] += v[e];
}

// rows_load through L2 only (data written by other SMs in this launch)
template <typename V, int VEC>
__device__ __forceinline__ void rows_load_l2(V (&out)[VEC], const V* p, bool full, int nvalid) {
    if (full) {
        using VT = typename RowsVec<V, VEC>::type;
        const VT v = __ldcg(reinterpret_cast<const VT*>(p));
        const V* e = reinterpret_cast<const V*>(&v);
#pragma unroll
        for (int i = 0; i < VEC; ++i) out[i] = e[i];
    } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i) out[i] = i < nvalid ? __ldcg(p + i) : V(0);
    }
}

template <typename V, int VEC>
__device__ __forceinline__ void rows_store(V* p, const V (&v)[VEC], bool full, int nvalid, bool accumulate) {
    if (full) {
        using VT = typename RowsVec<V, VEC>::type;
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

// Rows of a tile-row one task covers: all of them at T = 4 and 8; at T = 16
// and 32 a task is one group of 8 rows (G = T / 8 groups per tile-row, each
// its own work item), so its accumulators, item lists and occupancy are those
// of T = 8.  Groups of 8 rows walk each tile half as often as groups of 4:
// R-MAT scale 18, k = 64: 0.496 / 1.041 ms at T = 16 / 32 against 0.600 /
// 1.283 ms with groups of 4 (the merge-path kernel: 3.00 / 14.7 ms).
template <int T> constexpr int ROWS_R = T <= 8 ? T : 8;
// blocks of ROWS_WARPS warps per SM the register budget is written for
template <int T> constexpr int ROWS_BLOCKS = ROWS_R<T> == 4 ? 4 : 2;

// Packed per-row bit counts: FIELD bits per row (a row total over 32 lanes
// is at most 32*T: 128 fits 8 bits for T = 4; 256, 512 and 1024 take 16).
template <int T> struct RowsPack {
    static constexpr int FIELD = T == 4 ? 8 : 16;
    static constexpr int PER = 32 / FIELD;        // rows per 32-bit pack
    static constexpr int NP = ROWS_R<T> / PER;    // packs
    static constexpr uint32_t MASK = (1u << FIELD) - 1;
};

// The rows of lane's tile that its task covers.  T = 4 / 8: the whole tile as
// 64 bits, row r in byte r (T = 4: low nibble).  T = 16 / 32: rows
// R*g .. R*g+R-1 of group g, R*T/32 words read with 16-byte loads.
// bits(r): row r's word, bit T-1-c = column c.
template <int T> struct RowsWordNarrow {
    unsigned long long w = 0;
    __device__ __forceinline__ void load(const void* tiles, int j, int) {
        if constexpr (T == 4) {
            w = __ldg(static_cast<const unsigned int*>(tiles) + j);
        } else {
            const uint2 v = __ldg(static_cast<const uint2*>(tiles) + j);
            w = ((unsigned long long)v.y << 32) | v.x;
        }
    }
    __device__ __forceinline__ uint32_t bits(int r) const { return (uint32_t)(w >> (8 * r)) & ((1u << T) - 1u); }
};
template <int T> struct RowsWordWide {
    static constexpr int NW = ROWS_R<T> * T / 32;  // 32-bit words of a group: 4 (T = 16), 8 (T = 32)
    static_assert(NW % 4 == 0, "a group is whole 16-byte words");
    uint32_t w[NW] = {};
    __device__ __forceinline__ void load(const void* tiles, int j, int g) {
        // byte offset j*T*T/8 + g*NW*4: a multiple of 16
        const uint32_t* p = static_cast<const uint32_t*>(tiles) + (size_t)j * (T * T / 32) + (size_t)g * NW;
#pragma unroll
        for (int i = 0; i < NW / 4; ++i) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(p) + i);
            w[4 * i] = v.x;
            w[4 * i + 1] = v.y;
            w[4 * i + 2] = v.z;
            w[4 * i + 3] = v.w;
        }
    }
    __device__ __forceinline__ uint32_t bits(int r) const {
        if constexpr (T == 16) return (w[r >> 1] >> (16 * (r & 1))) & 0xffffu;
        else return w[r];
    }
};
template <int T>
using RowsWord = typename std::conditional<(T <= 8), RowsWordNarrow<T>, RowsWordWide<T>>::type;

}  // namespace

template <typename V>
struct SpmmRowsArgs {
    const int* colind;
    const void* tiles;
    const V* X;
    V* Y;
    long long ldx, ldy;
    int k;    // total columns
    int ncb;  // column blocks of (32 / IPW) * VEC columns
    const int4* tasks;  // (tile-row, first tile, end tile, slot or -1)
    int ntasks;
    int* state;   // [0] queue counter, [1] warps done, [2 + i*G + g] segments done of long row i, row group g
    const int4* long_rows;  // (tile-row, first slot, slots, 0)
    const int* slot_long;   // long row of every slot
    V* partials;  // slot x T x k
    int accumulate;
};

// The warp that finished the last segment of long row lr's row group (rows
// r0 .. r0+R-1 of its tile-row): those Y rows (+)= the row's slots added in
// segment order, over all k columns (every column block of the group has
// arrived); sub-group `sub` takes rows r0+sub, r0+sub+IPW, ...  SL slots in
// flight (2 with whole tile-rows, whose main loop needs the registers; 8 with
// 8-row groups at T = 16 / 32, whose long rows have the most slots), added
// in slot order; no unrolling of the outer loops (an out-of-line call
// measured slower).
template <int T, int IPW, bool FULL, typename V>
__device__ __forceinline__ void rows_long_reduce(const SpmmRowsArgs<V>& a, int lr, int lane, int r0) {
    constexpr int VEC = 16 / (int)sizeof(V);
    constexpr int LPI = 32 / IPW;
    constexpr int KC = LPI * VEC;
    constexpr int R = ROWS_R<T>;
    constexpr int SL = T >= 16 ? 8 : 2;
    const int sub = lane / LPI;
    const int4 L = __ldg(a.long_rows + lr);
    const long long stride = (long long)T * a.k;
#pragma unroll 1
    for (int cb = 0; cb < a.ncb; ++cb) {
        const int col = cb * KC + (lane % LPI) * VEC;
        const int nvalid = max(0, min(VEC, a.k - col));
        if (nvalid == 0) continue;
#pragma unroll 1
        for (int r = r0 + sub; r < r0 + R; r += IPW) {
            const V* src = a.partials + ((long long)L.y * T + r) * a.k + col;
            V tot[VEC];
#pragma unroll
            for (int e = 0; e < VEC; ++e) tot[e] = V(0);
            int q = 0;
#pragma unroll 1
            for (; q + SL - 1 < L.z; q += SL) {
                V v[SL][VEC];
#pragma unroll
                for (int u = 0; u < SL; ++u) rows_load_l2<V, VEC>(v[u], src + (q + u) * stride, FULL, nvalid);
#pragma unroll
                for (int u = 0; u < SL; ++u)
#pragma unroll
                    for (int e = 0; e < VEC; ++e) tot[e] += v[u][e];
            }
#pragma unroll 1
            for (; q < L.z; ++q) {
                V v0[VEC];
                rows_load_l2<V, VEC>(v0, src + q * stride, FULL, nvalid);
#pragma unroll
                for (int e = 0; e < VEC; ++e) tot[e] += v0[e];
            }
            rows_store<V, VEC>(a.Y + ((long long)L.x * T + r) * a.ldy + col, tot, FULL, nvalid,
                               a.accumulate != 0);
        }
    }
}

// VEC = 16 bytes of columns per lane; a warp loads IPW items (X rows) per
// instruction, LPI = 32/IPW lanes per item, so a column block is LPI*VEC
// columns (k = 64 FP32: two X rows per warp load).  FULL: every column
// vector is whole and 16-byte aligned (else per-element guarded loads).
// Work item wi = (column block, task, row group), the group fastest, so the
// G warps of one tile-row read its structure at about the same time.
template <int T, int IPW, bool FULL, typename V>
__global__ void __launch_bounds__(ROWS_WARPS * 32, ROWS_BLOCKS<T>)
spmm_rows_kernel(SpmmRowsArgs<V> a) {
    using P = RowsPack<T>;
    constexpr int R = ROWS_R<T>;  // rows per task
    constexpr int G = T / R;      // row groups per tile-row
    // a step of 32 tiles adds at most 32*T items to a row: more than a region
    // holds only at T >= 16, where such a step is appended in lane ranges
    constexpr bool SPLIT = 32 * T > ROWS_CAP;
    static_assert(T <= ROWS_CAP, "one tile's items of a row must fit an empty region");
    constexpr int VEC = 16 / (int)sizeof(V);
    constexpr int LPI = 32 / IPW;
    constexpr int KC = LPI * VEC;
    extern __shared__ int s_items[];  // per warp: R regions of ROWS_CAP items
    const int lane = threadIdx.x & 31;
    const int sub = lane / LPI;  // which item of an instruction this lane loads
    int* items = s_items + (threadIdx.x >> 5) * R * ROWS_CAP;
    const long long nwork = (long long)a.ntasks * a.ncb * G;
    const unsigned ldx = (unsigned)a.ldx;
    while (true) {
        int wi = 0;
        if (lane == 0) wi = atomicAdd(a.state, 1);
        wi = __shfl_sync(FULL_MASK, wi, 0);
        if (wi >= nwork) {
            // every warp fetches past the end exactly once; the last one to
            // count itself out leaves the state zeroed for the next launch
            if (lane == 0) {
                __threadfence();
                if (atomicAdd(a.state + 1, 1) == (int)(gridDim.x * ROWS_WARPS) - 1) {
                    a.state[0] = 0;
                    a.state[1] = 0;
                }
            }
            break;
        }
        // column block major: one pass over the tasks per block of X columns
        const int gi = G == 1 ? 0 : wi % G;
        const int wt = G == 1 ? wi : wi / G;
        const int cb = wt / a.ntasks, task = wt - cb * a.ntasks;
        const int4 t = __ldg(a.tasks + task);
        const int col = cb * KC + (lane % LPI) * VEC;
        const int nvalid = max(0, min(VEC, a.k - col));
        const bool active = nvalid > 0;
        const V* xc = a.X + col;
        V acc[R][VEC];
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int e = 0; e < VEC; ++e) acc[r][e] = V(0);

        int cnt[R];  // items in each row's region so far (warp-uniform)
#pragma unroll
        for (int r = 0; r < R; ++r) cnt[r] = 0;
        for (int j0 = t.y;; j0 += 32) {
            const bool more = j0 < t.z;  // warp-uniform
            const int j = j0 + lane;
            int tc = 0;
            RowsWord<T> w;
            if (more && j < t.z) {
                tc = __ldg(a.colind + j);
                w.load(a.tiles, j, gi);
            }
            // inclusive scan of the packed per-row counts of this step
            uint32_t inc[P::NP], own[P::NP];
#pragma unroll
            for (int p = 0; p < P::NP; ++p) {
                uint32_t c = 0;
#pragma unroll
                for (int q = 0; q < P::PER; ++q) c |= (uint32_t)__popc(w.bits(p * P::PER + q)) << (q * P::FIELD);
                own[p] = c;
                inc[p] = c;
#pragma unroll
                for (int s = 1; s < 32; s <<= 1) {
                    const uint32_t v = __shfl_up_sync(FULL_MASK, inc[p], s);
                    if (lane >= s) inc[p] += v;
                }
            }
            int tot[R];  // this step's items per row (warp-uniform)
            bool flush = !more, split = false;
#pragma unroll
            for (int p = 0; p < P::NP; ++p) {
                const uint32_t all = __shfl_sync(FULL_MASK, inc[p], 31);
#pragma unroll
                for (int q = 0; q < P::PER; ++q) {
                    const int r = p * P::PER + q;
                    tot[r] = (int)((all >> (q * P::FIELD)) & P::MASK);
                    flush |= cnt[r] + tot[r] > ROWS_CAP;
                    split |= tot[r] > ROWS_CAP;
                }
            }
            // the step's lanes in nsub ranges (one unless a row of the step
            // alone would overflow an empty region: then ROWS_CAP / T lanes each)
            int nsub = 1;
            if constexpr (SPLIT) {
                if (split) nsub = 32 * T / ROWS_CAP;
            }
            for (int sb = 0; sb < nsub; ++sb) {
                const int l0 = sb * (32 / nsub), l1 = l0 + 32 / nsub;  // lanes [l0, l1)
                uint32_t base[P::NP];  // packed counts of the lanes before l0
                int rt[R];             // the range's items per row
#pragma unroll
                for (int p = 0; p < P::NP; ++p) base[p] = 0;
#pragma unroll
                for (int r = 0; r < R; ++r) rt[r] = tot[r];
                if constexpr (SPLIT) {
                    if (nsub > 1) {  // warp-uniform
                        flush = false;
#pragma unroll
                        for (int p = 0; p < P::NP; ++p) {
                            base[p] = __shfl_sync(FULL_MASK, inc[p] - own[p], l0);
                            const uint32_t top = __shfl_sync(FULL_MASK, inc[p], l1 - 1) - base[p];
#pragma unroll
                            for (int q = 0; q < P::PER; ++q) {
                                const int r = p * P::PER + q;
                                rt[r] = (int)((top >> (q * P::FIELD)) & P::MASK);
                                flush |= cnt[r] + rt[r] > ROWS_CAP;
                            }
                        }
                    }
                }
                if (flush) {
                    // consume every row's region: sub-group `sub` takes items sub,
                    // sub+IPW, ... with ROWS_BATCH loads in flight per lane
                    if (active) {
#pragma unroll
                        for (int r = 0; r < R; ++r) {
                            const int* it = items + r * ROWS_CAP;
                            const int qb = cnt[r];
                            int q = sub;
                            for (; q + (ROWS_BATCH - 1) * IPW < qb; q += ROWS_BATCH * IPW) {
                                V xv[ROWS_BATCH][VEC];
#pragma unroll
                                for (int u = 0; u < ROWS_BATCH; ++u) {
                                    const unsigned xr = (unsigned)it[q + u * IPW];
                                    rows_load<V, VEC>(xv[u], xc + (size_t)xr * ldx, FULL, nvalid);
                                }
#pragma unroll
                                for (int u = 0; u < ROWS_BATCH; ++u) rows_add<V, VEC>(acc[r], xv[u]);
                            }
                            for (; q < qb; q += 4 * IPW) {  // the rest, four loads per lane per round
                                V xv[4][VEC];
#pragma unroll
                                for (int u = 0; u < 4; ++u) {
                                    if (q + u * IPW < qb) {
                                        rows_load<V, VEC>(xv[u], xc + (size_t)(unsigned)it[q + u * IPW] * ldx, FULL,
                                                          nvalid);
                                    } else {
#pragma unroll
                                        for (int e = 0; e < VEC; ++e) xv[u][e] = V(0);
                                    }
                                }
#pragma unroll
                                for (int u = 0; u < 4; ++u) rows_add<V, VEC>(acc[r], xv[u]);
                            }
                        }
                    }
#pragma unroll
                    for (int r = 0; r < R; ++r) cnt[r] = 0;
                    __syncwarp();
                }
                if (!more) break;
                // append the range's items to the row regions: X row index of
                // every set bit, in lane then column order
                if (lane >= l0 && lane < l1) {
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const int p = r / P::PER, q = r % P::PER;
                        int pos = r * ROWS_CAP + cnt[r] +
                                  (int)((((inc[p] - own[p]) - base[p]) >> (q * P::FIELD)) & P::MASK);
                        uint32_t bits = w.bits(r);
                        while (bits) {
                            const int b = 31 - __clz(bits);  // ascending column c = T-1-b
                            bits ^= 1u << b;
                            items[pos++] = tc * T + (T - 1 - b);
                        }
                    }
                }
#pragma unroll
                for (int r = 0; r < R; ++r) cnt[r] += rt[r];
                __syncwarp();
            }
            if (!more) break;
        }
        // combine the IPW sub-groups (fixed butterfly order)
#pragma unroll
        for (int m = LPI; m < 32; m <<= 1)
#pragma unroll
            for (int r = 0; r < R; ++r)
#pragma unroll
                for (int e = 0; e < VEC; ++e) acc[r][e] += __shfl_xor_sync(FULL_MASK, acc[r][e], m);
        const bool writer = active && sub == 0;
        const int r0 = gi * R;  // first row of the tile-row this task covers
        if (t.w < 0) {
            if (writer) {
#pragma unroll
                for (int r = 0; r < R; ++r)
                    rows_store<V, VEC>(a.Y + ((long long)t.x * T + r0 + r) * a.ldy + col, acc[r], FULL, nvalid,
                                       a.accumulate != 0);
            }
            continue;
        }
        // a segment of a long row: its partial rows to the slot, then count in
        V* dst = a.partials + ((long long)t.w * T + r0) * a.k + col;
        if (writer) {
#pragma unroll
            for (int r = 0; r < R; ++r) rows_store<V, VEC>(dst + (long long)r * a.k, acc[r], FULL, nvalid, false);
        }
        __threadfence();
        __syncwarp();
        int lr = 0, last = 0;
        if (lane == 0) {
            lr = __ldg(a.slot_long + t.w);
            // arrivals per (long row, row group): each segment once per column block
            last = atomicAdd(a.state + 2 + lr * G + gi, 1) == __ldg(a.long_rows + lr).z * a.ncb - 1;
        }
        if (!__shfl_sync(FULL_MASK, last, 0)) continue;
        // the group's last segment: its Y rows (+)= its slots added in segment order
        lr = __shfl_sync(FULL_MASK, lr, 0);
        __threadfence();
        rows_long_reduce<T, IPW, FULL, V>(a, lr, lane, r0);
        if (lane == 0) a.state[2 + lr * G + gi] = 0;
    }
}

// ---- plan ---------------------------------------------------------------------------
// Longest task in tiles: a fixed share of one resident warp's part of the
// tile visits (4 blocks of 8 warps per SM with 4-row tasks, 2 with 8-row
// tasks), so that the queue stays balanced at every graph size.  The shares,
// 30% with 4-row tasks and 20% with 8-row tasks, were the best of 20/30/40%
// on R-MAT scales 16-20 with k = 64 and 128 on GB300; 40% fell off a cliff
// (the queue's end waits on long segments).  At T = 16 / 32 a task's tiles
// are walked once per row group, so the visits are nt x T/8.
int spmm_rows_seg(int T, long long nt, int num_sms) {
    const int R = T <= 8 ? T : ROWS_R<32>;
    const long long visits = nt * (T / R);
    const long long warps = (long long)std::max(num_sms, 1) * (R == 4 ? 4 : 2) * ROWS_WARPS;
    const long long pct = R == 4 ? 30 : 20;
    return (int)std::min(8192LL, std::max(128LL, visits * pct / (100 * warps)));
}

// Set bits of every tile-row: one warp per tile-row (grid-stride), popc of
// its tiles' 32-bit words (the unused bits of a tile are zero).
__global__ void tile_row_bits_kernel(const int* __restrict__ rowptr, const uint32_t* __restrict__ words, int nb,
                                     int wpt, long long* __restrict__ bits) {
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nb; r += nwarps) {
        const long long b = (long long)rowptr[r] * wpt, e = (long long)rowptr[r + 1] * wpt;
        long long c = 0;
        for (long long k = b + lane; k < e; k += 32) c += __popc(__ldg(words + k));
#pragma unroll
        for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(FULL_MASK, c, o);
        if (lane == 0) bits[r] = c;
    }
}

b2sr_status spmm_rows_plan_create(const int* d_rowptr, const void* d_tiles, int nb, int T, int num_sms,
                                  SpmmRowsPlan* out, cudaStream_t s) {
    std::vector<int> rp((size_t)nb + 1);
    cudaError_t e = cudaMemcpyAsync(rp.data(), d_rowptr, sizeof(int) * rp.size(), cudaMemcpyDeviceToHost, s);
    // T = 16 / 32: the set bits of every tile-row.  A row group holding hub
    // rows carries far more set bits than its tiles suggest (R-MAT scale 18,
    // T = 32: ~9.3 K X-row loads for one warp in a tile-bounded segment of
    // tile-row 0, against 3.1 K set bits per resident warp on average),
    // so there segments are also bounded by set bits: at most one resident
    // warp's average share of all the bits (with the queue ordered by set
    // bits and the long rows reduced per row group: R-MAT scale 18, k = 64,
    // 0.295 / 0.377 ms at T = 16 / 32 against 0.484 / 1.027 ms with
    // tile-bounded segments).
    const bool by_bits = T >= 16 && nb > 0;
    std::vector<long long> rbits;
    if (e == cudaSuccess && by_bits) {
        long long* d_bits = static_cast<long long*>(dev_alloc(sizeof(long long) * (size_t)nb));
        if (!d_bits) return B2SR_ERR_ALLOC;
        rbits.resize((size_t)nb);
        const long long blocks = std::min<long long>(((long long)nb * 32 + 255) / 256, 65535LL * 8);
        tile_row_bits_kernel<<<(unsigned)blocks, 256, 0, s>>>(d_rowptr, static_cast<const uint32_t*>(d_tiles), nb,
                                                                T * T / 32, d_bits);
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(rbits.data(), d_bits, sizeof(long long) * (size_t)nb, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        dev_free(d_bits);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return B2SR_ERR_CUDA;
    }
    const int seg = spmm_rows_seg(T, rp[nb], num_sms);
    long long seg_bits = 0;
    if (by_bits) {
        long long total = 0;
        for (long long v : rbits) total += v;
        const long long warps = (long long)std::max(num_sms, 1) * ROWS_BLOCKS<32> * ROWS_WARPS;
        seg_bits = std::max(1024LL, total / warps);
    }
    std::vector<int4> tasks, longs;
    std::vector<long long> work;  // estimated set bits of each task (T = 16 / 32)
    tasks.reserve((size_t)nb + 16);
    int nslots = 0;
    for (int i = 0; i < nb; ++i) {
        const int b0 = rp[i], m = rp[i + 1] - b0;
        int nseg = (m + seg - 1) / seg;  // near-equal segments of at most seg tiles
        if (by_bits) nseg = (int)std::min<long long>(m, std::max<long long>(nseg, (rbits[i] + seg_bits - 1) / seg_bits));
        if (nseg <= 1) {
            tasks.push_back(make_int4(i, b0, b0 + m, -1));
            if (by_bits) work.push_back(rbits[i]);
        } else {
            longs.push_back(make_int4(i, nslots, nseg, 0));
            for (int q = 0; q < nseg; ++q) {
                const int t0 = b0 + (int)((long long)m * q / nseg), t1 = b0 + (int)((long long)m * (q + 1) / nseg);
                tasks.push_back(make_int4(i, t0, t1, nslots + q));
                if (by_bits) work.push_back((long long)((double)rbits[i] * (t1 - t0) / m));
            }
            nslots += nseg;
        }
    }
    // Queue order.  T = 4: tasks of at least a quarter of a segment first,
    // then the rest, each class in tile-row order, so the queue ends on short
    // tasks while tile-rows that share X rows (the blocks of a batched graph)
    // still run together: R-MAT scale 18 / 20 as fast as longest first, and
    // 512 stacked ER graphs 1.86 ms against 2.85 ms longest first (2.61 ms in
    // row order with fixed segments).  T = 8: longest first (R-MAT scale 18:
    // 0.233 against 0.268 ms with the split).  T = 16 / 32: most set bits
    // first.
    if (by_bits) {
        std::vector<int> order(tasks.size());
        for (size_t q = 0; q < order.size(); ++q) order[q] = (int)q;
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return work[x] > work[y]; });
        std::vector<int4> sorted(tasks.size());
        for (size_t q = 0; q < order.size(); ++q) sorted[q] = tasks[order[q]];
        tasks.swap(sorted);
    } else if (T == 4) {
        std::stable_partition(tasks.begin(), tasks.end(), [seg](const int4& t) { return 4 * (t.z - t.y) >= seg; });
    } else {
        std::stable_sort(tasks.begin(), tasks.end(),
                         [](const int4& x, const int4& y) { return x.z - x.y > y.z - y.y; });
    }
    SpmmRowsPlan p;
    p.groups = T / (T <= 8 ? T : ROWS_R<32>);
    p.ntasks = (int)tasks.size();
    p.nlong = (int)longs.size();
    p.nslots = nslots;
    std::vector<int> slot_long((size_t)std::max(nslots, 1), 0);
    for (int i = 0; i < p.nlong; ++i)
        for (int q = 0; q < longs[i].z; ++q) slot_long[(size_t)longs[i].y + q] = i;
    p.d_tasks = static_cast<int4*>(dev_alloc(sizeof(int4) * (size_t)std::max(p.ntasks, 1)));
    p.d_long = static_cast<int4*>(dev_alloc(sizeof(int4) * (size_t)std::max(p.nlong, 1)));
    p.d_slot_long = static_cast<int*>(dev_alloc(sizeof(int) * slot_long.size()));
    if (!p.d_tasks || !p.d_long || !p.d_slot_long) {
        spmm_rows_plan_free(&p);
        return B2SR_ERR_ALLOC;
    }
    e = cudaSuccess;
    if (p.ntasks) e = cudaMemcpy(p.d_tasks, tasks.data(), sizeof(int4) * (size_t)p.ntasks, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && p.nlong)
        e = cudaMemcpy(p.d_long, longs.data(), sizeof(int4) * (size_t)p.nlong, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(p.d_slot_long, slot_long.data(), sizeof(int) * slot_long.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        spmm_rows_plan_free(&p);
        return B2SR_ERR_CUDA;
    }
    *out = p;
    return B2SR_SUCCESS;
}

void spmm_rows_plan_free(SpmmRowsPlan* p) {
    dev_free(p->d_tasks);
    dev_free(p->d_long);
    dev_free(p->d_slot_long);
    p->d_tasks = nullptr;
    p->d_long = nullptr;
    p->d_slot_long = nullptr;
}

// Items per warp load.  rhs_block > 0 (FP32 columns; half as many FP64
// columns) fixes the column block 32/IPW lanes x 16 bytes; 0 takes the
// largest power of two IPW (at most 8) whose block still covers k.
static int rows_ipw(int elem_bytes, int k, int rhs_block) {
    const int vec = 16 / elem_bytes;
    if (rhs_block > 0) {
        const int cols = rhs_block * 4 / elem_bytes;  // columns of this element size
        int ipw = 1;
        while (ipw < 8 && (32 / (2 * ipw)) * vec >= cols) ipw *= 2;
        return ipw;
    }
    int ipw = 1;
    while (ipw < 8 && (32 / (2 * ipw)) * vec >= k) ipw *= 2;
    return ipw;
}

size_t spmm_rows_scratch_bytes(const SpmmRowsPlan& p, int T, int elem_bytes, int k) {
    return (size_t)std::max(p.nslots, 1) * T * (size_t)k * elem_bytes;
}

size_t spmm_rows_state_bytes(const SpmmRowsPlan& p) { return sizeof(int) * (2 + (size_t)p.nlong * p.groups); }

template <int T, int IPW, bool FULL, typename V>
static b2sr_status run_rows(SpmmRowsArgs<V> a, const SpmmRowsPlan& p, int num_sms, cudaStream_t s) {
    constexpr int SMEM = ROWS_WARPS * ROWS_R<T> * ROWS_CAP * (int)sizeof(int);
    // per device: the attribute is set on every launch (cheap), the occupancy once
    cudaError_t e = cudaFuncSetAttribute(spmm_rows_kernel<T, IPW, FULL, V>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return B2SR_ERR_CUDA;
    }
    static int blocks_per_sm = 0;  // per instantiation; the device's SM count scales it
    if (blocks_per_sm == 0) {
        int n = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, spmm_rows_kernel<T, IPW, FULL, V>, ROWS_WARPS * 32,
                                                          SMEM);
        if (e != cudaSuccess) {
            set_cuda_error(e);
            return B2SR_ERR_CUDA;
        }
        blocks_per_sm = std::max(n, 1);
    }
    const long long nwork = (long long)a.ntasks * a.ncb * (T / ROWS_R<T>);
    const long long want = (nwork + ROWS_WARPS - 1) / ROWS_WARPS;
    const int grid = (int)std::max(1LL, std::min<long long>((long long)num_sms * blocks_per_sm, want));
    // the queue counter is a 32-bit int that ends at nwork + one fetch per
    // warp, and a long row's arrivals count to its slots x ncb
    if (nwork + (long long)grid * ROWS_WARPS >= 0x7fffffffLL) return B2SR_ERR_NOT_SUPPORTED;
    kernel_timer_mark(s, true);
    spmm_rows_kernel<T, IPW, FULL, V><<<grid, ROWS_WARPS * 32, SMEM, s>>>(a);
    kernel_timer_mark(s, false);
    B2SR_LAUNCH_CHECK();
    add_launch_count(1);
    return B2SR_SUCCESS;
}

template <int T, typename V>
static b2sr_status rows_dispatch(const SpmmRowsArgs<V>& a, int ipw, bool full, const SpmmRowsPlan& p, int num_sms,
                                 cudaStream_t s) {
#define B2SR_ROWS_IPW(I)                                                   \
    if (ipw == I) return full ? run_rows<T, I, true, V>(a, p, num_sms, s) \
                              : run_rows<T, I, false, V>(a, p, num_sms, s);
    B2SR_ROWS_IPW(1) B2SR_ROWS_IPW(2) B2SR_ROWS_IPW(4) B2SR_ROWS_IPW(8)
#undef B2SR_ROWS_IPW
    return B2SR_ERR_INVALID_VALUE;
}

template <typename V>
b2sr_status spmm_rows_launch(const MatView& A, const SpmmRowsPlan& p, const V* X, long long ldx, V* Y,
                             long long ldy, int k, int rhs_block, int accumulate, void* scratch, int* state,
                             int num_sms, cudaStream_t s) {
    constexpr int VEC = 16 / (int)sizeof(V);
    if (ldx > 0x7fffffffLL) return B2SR_ERR_NOT_SUPPORTED;
    const int ipw = rows_ipw((int)sizeof(V), k, rhs_block);
    const int KC = (32 / ipw) * VEC;
    SpmmRowsArgs<V> a;
    a.colind = A.colind;
    a.tiles = A.tiles;
    a.X = X;
    a.Y = Y;
    a.ldx = ldx;
    a.ldy = ldy;
    a.k = k;
    a.ncb = (k + KC - 1) / KC;
    a.tasks = p.d_tasks;
    a.ntasks = p.ntasks;
    a.state = state;
    a.long_rows = p.d_long;
    a.slot_long = p.d_slot_long;
    a.partials = static_cast<V*>(scratch);
    a.accumulate = accumulate;
    // whole 16-byte column vectors everywhere: X, Y aligned, row strides and k multiples of VEC
    const bool full = ((uintptr_t)X % 16 == 0) && ((uintptr_t)Y % 16 == 0) && (ldx % VEC == 0) &&
                      (ldy % VEC == 0) && (k % VEC == 0);
    if (A.T == 4) return rows_dispatch<4, V>(a, ipw, full, p, num_sms, s);
    if (A.T == 8) return rows_dispatch<8, V>(a, ipw, full, p, num_sms, s);
    if (A.T == 16) return rows_dispatch<16, V>(a, ipw, full, p, num_sms, s);
    if (A.T == 32) return rows_dispatch<32, V>(a, ipw, full, p, num_sms, s);
    return B2SR_ERR_INVALID_VALUE;
}

template b2sr_status spmm_rows_launch<float>(const MatView&, const SpmmRowsPlan&, const float*, long long, float*,
                                             long long, int, int, int, void*, int*, int, cudaStream_t);
template b2sr_status spmm_rows_launch<double>(const MatView&, const SpmmRowsPlan&, const double*, long long,
                                              double*, long long, int, int, int, void*, int*, int, cudaStream_t);

}  // namespace b2sr
