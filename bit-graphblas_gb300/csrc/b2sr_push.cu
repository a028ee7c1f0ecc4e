// Direction-optimised bit-vector products: "push" over the transposed B2SR.
//
// Tile-row c of A^T holds the tiles of A's tile-column c with rows and columns
// swapped: word cc of the A^T tile in tile-column tr has bit T-1-r set iff
// A[tr*T + r][c*T + cc] = 1.  So for a sparse x (a BFS frontier) the product
// needs only the tile-rows of A^T whose x word is non-zero:
//   bin_bin_bin:  y[tr] |= OR of the A^T words cc whose x bit T-1-cc is set
//   counts:       y[tr*T + r] += number of those words with bit T-1-r set
// OR and integer sums do not depend on order, so the result equals the pull
// kernels' bit for bit.  The reference has no push form: its BFS multiplies
// every tile-row each level (bmv_eval/backend/bsrbmv.cu:1083-1229).
//
// A classify kernel lists the active tile-columns as work items of at most
// CHUNK tiles (hub columns split across warps) and counts their tiles; in
// auto mode the push kernel runs when that count is below push_percent(T)% of nt and
// the pull kernels (launched after it) otherwise -- both read the count on the
// device, so nothing waits on the host and the sequence can be captured.
#include "b2sr_common.cuh"
#include "b2sr_spmv_impl.cuh"

#include <type_traits>

namespace b2sr {

namespace {

// Tiles per lane and per work item: a work item is one warp pass.
template <int T> struct PushU { static constexpr int value = T <= 8 ? 8 : T == 16 ? 4 : 1; };
template <int T> struct PushChunk { static constexpr int value = 32 * PushU<T>::value; };
constexpr int MIN_CHUNK = 32;

struct PushArgs {
    const int* t_rowptr;
    const int* t_colind;
    const void* t_tiles;
    const void* x;
    void* y;
    const void* mask;
    const int* ctl;     // [0] work items, [1] tiles of A^T under active x words
    const int4* items;  // (first tile, end tile, x word, 0): no dependent loads before the tiles
    int mode;
    int pct;
    long long nt;
    int* hint;  // auto direction: where the decision is recorded for the next call (1 push, 2 pull), or null
};

// One thread per tile-column of A: lists the work items of active columns.
// Also zeroes y (y_n elements of type Y; none with accumulate) before the push
// kernel adds into it.  The counters take one atomic per block (a block scan
// of the warps' totals), not one per warp: same-address atomics serialise.
constexpr int CLASSIFY_THREADS = 256;

// COUNT: only the tile count, into ctl[1] (no list, y untouched); the last
// block to finish (ctl[2] counts them) records the direction for a share of
// pct% of nt in *hint and leaves ctl zeroed for the next launch.
template <int T, typename Y, bool COUNT>
__global__ void __launch_bounds__(CLASSIFY_THREADS)
    push_classify_kernel(const void* __restrict__ x, int nbc, const int* __restrict__ t_rowptr, int* __restrict__ ctl,
                         int4* __restrict__ items, Y* __restrict__ y, long long y_n, long long nt, int pct,
                         int* hint) {
    using W = typename TileWord<T>::type;
    constexpr int CH = PushChunk<T>::value;
    constexpr int NW = CLASSIFY_THREADS / 32;
    __shared__ int s_items[NW], s_work[NW], s_base;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (!COUNT)
        for (long long i = c; i < y_n; i += (long long)gridDim.x * blockDim.x) y[i] = Y(0);
    const int xw = c < nbc ? (int)__ldg(static_cast<const W*>(x) + c) : 0;
    const bool active = xw != 0;
    const int b = active ? __ldg(t_rowptr + c) : 0;
    const int len = active ? __ldg(t_rowptr + c + 1) - b : 0;
    const int nch = (len + CH - 1) / CH;
    int incl = nch, work = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(FULL_MASK, incl, o);
        if (lane >= o) incl += v;
        work += __shfl_xor_sync(FULL_MASK, work, o);
    }
    if (lane == 31) {
        s_items[warp] = incl;
        s_work[warp] = work;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int tot = 0, wk = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            const int n = s_items[w];
            s_items[w] = tot;  // exclusive prefix over the block's warps
            tot += n;
            wk += s_work[w];
        }
        if (COUNT) {
            if (wk) atomicAdd(ctl + 1, wk);
            __threadfence();
            if (atomicAdd(ctl + 2, 1) == (int)gridDim.x - 1) {
                __threadfence();
                const long long active = atomicAdd(ctl + 1, 0);
                *reinterpret_cast<volatile int*>(hint) = active * 100 < nt * pct ? 1 : 2;
                ctl[1] = 0;
                ctl[2] = 0;
            }
        } else {
            s_base = tot ? atomicAdd(ctl, tot) : 0;
            if (wk) atomicAdd(ctl + 1, wk);
        }
    }
    if (COUNT) return;
    __syncthreads();
    if (nch == 0) return;
    const int base = s_base + s_items[warp] + incl - nch;
    for (int k = 0; k < nch; ++k) {
        const int first = b + k * CH;
        items[base + k] = make_int4(first, first + CH < b + len ? first + CH : b + len, xw, 0);
    }
}

template <int T>
__device__ __forceinline__ void or_word(void* y, int tr, uint32_t m) {
    if constexpr (T == 32) {
        atomicOr(static_cast<unsigned int*>(y) + tr, m);
    } else {
        // 32-bit atomic on the aligned word holding y's word tr (1 or 2
        // bytes); the other bytes of that word are OR-ed with zero
        const uintptr_t p = reinterpret_cast<uintptr_t>(static_cast<typename TileWord<T>::type*>(y) + tr);
        atomicOr(reinterpret_cast<unsigned int*>(p & ~(uintptr_t)3), m << (8 * (unsigned)(p & 3)));
    }
}

// One warp per work item, U tiles per lane loaded before any is used.
template <int T, int KIND>
__global__ void __launch_bounds__(256) push_kernel(PushArgs a) {
    griddep_wait();  // launched behind the classify kernel: its counters and list
    const bool chosen = push_chosen(a.ctl, a.mode, a.nt, a.pct);
    if (a.hint && blockIdx.x == 0 && threadIdx.x == 0) *reinterpret_cast<volatile int*>(a.hint) = chosen ? 1 : 2;
    if (!chosen) return;
    using W = typename TileWord<T>::type;
    constexpr int U = PushU<T>::value;
    const int lane = threadIdx.x & 31;
    const int nitems = a.ctl[0];
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    const W* t_tiles = static_cast<const W*>(a.t_tiles);
    for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < nitems; i += nwarps) {
        const int4 it = a.items[i];
        const uint32_t xw = (uint32_t)it.z;
        const int e = it.y;
        int tr[U];
        TileBits<T> tb[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int j = it.x + lane + 32 * u;
            tr[u] = -1;
            if (j < e) {
                tr[u] = __ldg(a.t_colind + j);
                tb[u].load(t_tiles, j);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (tr[u] < 0) continue;
            if constexpr (KIND <= 1) {
                uint32_t m = 0;
#pragma unroll
                for (int cc = 0; cc < T; ++cc)
                    if ((xw >> (T - 1 - cc)) & 1u) m |= tb[u].row(cc);
                if (KIND == 1 && m) m &= ~(uint32_t)__ldg(static_cast<const W*>(a.mask) + tr[u]);
                if (m) or_word<T>(a.y, tr[u], m);
            } else {
                uint32_t cols[T];  // word cc if x bit T-1-cc is set, else 0
#pragma unroll
                for (int cc = 0; cc < T; ++cc) cols[cc] = ((xw >> (T - 1 - cc)) & 1u) ? tb[u].row(cc) : 0u;
#pragma unroll
                for (int r = 0; r < T; ++r) {
                    int cnt = 0;
#pragma unroll
                    for (int cc = 0; cc < T; ++cc) cnt += (int)((cols[cc] >> (T - 1 - r)) & 1u);
                    if (cnt) {
                        const size_t o = (size_t)tr[u] * T + r;
                        if constexpr (KIND == 2) atomicAdd(static_cast<int*>(a.y) + o, cnt);
                        else atomicAdd(static_cast<float*>(a.y) + o, (float)cnt);
                    }
                }
            }
        }
    }
}

template <int T, int KIND>
b2sr_status run_push(PushArgs a, int* ctl, int4* items, int nbc, long long y_n, bool timed, int num_sms,
                     cudaStream_t s) {
    // y's element: the tile word (bits), int32 or float (counts)
    using Y = typename std::conditional<KIND <= 1, typename TileWord<T>::type,
                                        typename std::conditional<KIND == 2, int, float>::type>::type;
    const long long cover = (long long)num_sms * 8 * 256;
    const long long zero_threads = y_n < cover ? y_n : cover;  // grid-stride over y
    const long long threads = nbc > zero_threads ? nbc : zero_threads;
    if (threads > 0) {
        push_classify_kernel<T, Y, false><<<(unsigned)((threads + CLASSIFY_THREADS - 1) / CLASSIFY_THREADS),
                                            CLASSIFY_THREADS, 0, s>>>(a.x, nbc, a.t_rowptr, ctl, items,
                                                                      static_cast<Y*>(a.y), y_n, 0, 0, nullptr);
        B2SR_LAUNCH_CHECK();
    }
    const int launches = threads > 0 ? 1 : 0;
    if (timed) kernel_timer_mark(s, true);
    B2SR_CUDA_TRY(launch_dependent(push_kernel<T, KIND>, (unsigned)(num_sms * 8), 256u, s, a));
    if (timed && a.mode == 2) kernel_timer_mark(s, false);
    add_launch_count(launches + 1);
    return B2SR_SUCCESS;
}

template <int T>
b2sr_status push_kind(int kind, const PushArgs& a, int* ctl, int4* items, int nbc, long long y_n, int num_sms,
                      cudaStream_t s) {
    switch (kind) {
        case 0: return run_push<T, 0>(a, ctl, items, nbc, y_n, true, num_sms, s);
        case 1: return run_push<T, 1>(a, ctl, items, nbc, y_n, true, num_sms, s);
        case 2: return run_push<T, 2>(a, ctl, items, nbc, y_n, true, num_sms, s);
        case 3: return run_push<T, 3>(a, ctl, items, nbc, y_n, true, num_sms, s);
    }
    return B2SR_ERR_INVALID_VALUE;
}

constexpr size_t CTL_BYTES = 256;

}  // namespace

size_t push_scratch_bytes(int nbc, long long nt) {
    // items: at most one per active column plus one per MIN_CHUNK tiles
    return CTL_BYTES + sizeof(int4) * ((size_t)(nbc > 0 ? nbc : 0) + (size_t)(nt / MIN_CHUNK) + 1);
}

b2sr_status launch_push(const MatView& At, int kind, int mode, const void* x, void* y, const void* mask,
                        int accumulate, size_t y_bytes, long long nt, void* scratch, int num_sms,
                        PushLink* link, int* hint, cudaStream_t s) {
    if (kind < 0 || kind > 3 || (mode != 1 && mode != 2)) return B2SR_ERR_INVALID_VALUE;
    int* ctl = static_cast<int*>(scratch);
    int4* items = reinterpret_cast<int4*>(static_cast<char*>(scratch) + CTL_BYTES);
    B2SR_CUDA_TRY(cudaMemsetAsync(ctl, 0, 2 * sizeof(int), s));
    PushArgs a;
    a.t_rowptr = At.rowptr;
    a.t_colind = At.colind;
    a.t_tiles = At.tiles;
    a.x = x;
    a.y = y;
    a.mask = mask;
    a.ctl = ctl;
    a.items = items;
    a.mode = mode;
    a.pct = push_percent(At.T);
    a.nt = nt;
    a.hint = hint;
    if (link) {
        link->ctl = ctl;
        link->nt = nt;
        link->pct = a.pct;
    }
    const int nbc = At.nb;  // A's tile-columns are A^T's tile-rows
    const long long y_n = accumulate ? 0 : (long long)(y_bytes / (kind <= 1 ? (size_t)word_bytes(At.T) : 4));
    switch (At.T) {
        case 4: return push_kind<4>(kind, a, ctl, items, nbc, y_n, num_sms, s);
        case 8: return push_kind<8>(kind, a, ctl, items, nbc, y_n, num_sms, s);
        case 16: return push_kind<16>(kind, a, ctl, items, nbc, y_n, num_sms, s);
        case 32: return push_kind<32>(kind, a, ctl, items, nbc, y_n, num_sms, s);
    }
    return B2SR_ERR_INVALID_VALUE;
}

template <int T>
static void launch_count(const MatView& At, const void* x, long long nt, int* state, int* hint, cudaStream_t s) {
    const int nbc = At.nb;
    push_classify_kernel<T, int, true><<<(unsigned)((nbc + CLASSIFY_THREADS - 1) / CLASSIFY_THREADS),
                                         CLASSIFY_THREADS, 0, s>>>(x, nbc, At.rowptr, state, nullptr, nullptr, 0,
                                                                   nt, push_percent(T), hint);
}

b2sr_status launch_direction_count(const MatView& At, const void* x, long long nt, int* state, int* hint,
                                   cudaStream_t s) {
    if (At.nb <= 0) return B2SR_SUCCESS;
    switch (At.T) {
        case 4: launch_count<4>(At, x, nt, state, hint, s); break;
        case 8: launch_count<8>(At, x, nt, state, hint, s); break;
        case 16: launch_count<16>(At, x, nt, state, hint, s); break;
        case 32: launch_count<32>(At, x, nt, state, hint, s); break;
        default: return B2SR_ERR_INVALID_VALUE;
    }
    B2SR_LAUNCH_CHECK();
    return B2SR_SUCCESS;
}

}  // namespace b2sr
