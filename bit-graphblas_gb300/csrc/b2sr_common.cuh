// Shared definitions of the B2SR library: tile word types, the matrix object,
// launch helpers and error plumbing.  Internal header (the public ABI is
// include/b2sr.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <climits>
#include <cstddef>
#include <deque>
#include <mutex>
#include <vector>

#include "../../include/b2sr.h"

namespace b2sr {

// Tile word type per tile size.  T = 4 keeps one byte per tile row with the
// row in the low nibble, as the reference's ToBit4Col does
// (bmv_eval/backend/bsrbmv.cu:33-62).
template <int T> struct TileWord;
template <> struct TileWord<4> { using type = uint8_t; };
template <> struct TileWord<8> { using type = uint8_t; };
template <> struct TileWord<16> { using type = uint16_t; };
template <> struct TileWord<32> { using type = uint32_t; };

template <int T> struct Log2;
template <> struct Log2<4> { static constexpr int value = 2; };
template <> struct Log2<8> { static constexpr int value = 3; };
template <> struct Log2<16> { static constexpr int value = 4; };
template <> struct Log2<32> { static constexpr int value = 5; };

inline int word_bytes(int T) { return T <= 8 ? 1 : T / 8; }
inline bool valid_tile(int T) { return T == 4 || T == 8 || T == 16 || T == 32; }

constexpr unsigned FULL_MASK = 0xffffffffu;

// Merge-path coordinate: `row` row-end items and `tile` tiles consumed.
struct Coord {
    int row;
    int tile;
};

// Launch shape of a merge-path multiply.
struct LaunchShape {
    int threads = 256;
    int items = 8;
    int ctas_per_sm = 0;
    int algorithm = 0;  // 0 auto, 1 merge-path, 2 row-binned
    int gather = 0;     // row-binned x gathers: 0 auto, 1 ld.global, 2 texture, 3 set columns only
    int rhs_block = 0;  // dense-RHS columns per warp pass (FP32 count; 0: narrowest covering k)
    int direction = 0;  // bit-vector variants: 0 pull, 1 auto (push for sparse x), 2 push
};

// Row-binned plan of a matrix (b2sr_rowbin.cu): tasks grouped by bin, the
// long rows' segment bookkeeping, and per-bin task/warp offsets.
struct RowBinPlan {
    int4* d_tasks = nullptr;
    int4* d_long = nullptr;
    int ntasks = 0, nlong = 0, nslots = 0;
    int nlong_short = 0;  // long rows with few slots, listed first in d_long
    int task_off[7] = {0, 0, 0, 0, 0, 0, 0};
    int warp_off[7] = {0, 0, 0, 0, 0, 0, 0};
};

// Row-task SpMM plan (b2sr_spmm_rows.cu, T = 4 and 8): one task per
// tile-row in row order, long rows cut into segments with partial slots.
struct SpmmRowsPlan {
    int4* d_tasks = nullptr;
    int4* d_long = nullptr;      // (tile-row, first slot, slots, 0)
    int* d_slot_long = nullptr;  // long row of every slot
    int ntasks = 0, nlong = 0, nslots = 0;
    int groups = 1;              // row groups per tile-row (T / rows per task)
};

// Per-variant cached launch data of a matrix: the grid and the merge-path
// start coordinate of every CTA (grid + 1 entries, device).
struct LaunchPlan {
    LaunchShape shape;
    int grid = 0;
    Coord* d_starts = nullptr;
};

}  // namespace b2sr

// The opaque handle of the C ABI.
struct b2sr_matrix {
    int nrows = 0, ncols = 0, T = 0;
    int nb = 0, nbc = 0, nt = 0;
    long long nnz = 0;
    int* rowptr = nullptr;
    int* colind = nullptr;
    void* tiles = nullptr;
    bool owns = false;
    int device = 0;
    int num_sms = 0;
    b2sr::LaunchShape shapes[4];
    b2sr::LaunchPlan plans[4];
    b2sr::LaunchPlan spmm_plan;  // chunk starts of the SpMM work queue
    b2sr::RowBinPlan rowbin;     // bin_full_full / multi-frontier row-binned plan
    bool rowbin_ready = false;
    b2sr::RowBinPlan rowbin_bits;  // the bit-vector kernels' plan
    bool rowbin_bits_ready = false;
    b2sr::SpmmRowsPlan spmm_rows;  // row-task SpMM plan (T = 4, 8)
    bool spmm_rows_ready = false;
    // Per-stream scratch (carries, partials, queue counter), grown on demand
    // and reused: calls on one stream are ordered, so they can share it.
    struct StreamScratch {
        cudaStream_t stream;
        void* ptr;
        size_t bytes;
    };
    std::mutex scratch_mu;
    std::vector<StreamScratch> scratch;
    // Per-stream counters of the row-task SpMM kernel (work queue, long-row
    // arrivals): zeroed when allocated, left zeroed by every launch, and
    // used by nothing else.
    std::vector<StreamScratch> spmm_state;
    // Auto direction outside stream captures: the device's last decision per
    // bit-vector kind (0 none yet, 1 push, 2 pull) in mapped host memory, read
    // by the next call as a hint; and per stream a side stream with two events
    // and a zeroed counter for the decision-only count beside a hinted pull.
    int* auto_hint = nullptr;
    struct AutoSide {
        cudaStream_t stream;
        cudaStream_t side;
        cudaEvent_t fork, join;
        int* state;
    };
    std::deque<AutoSide> auto_side;  // a deque: entries stay put while others are added
    // Buffers replaced by larger or rebuilt ones.  A CUDA graph captured
    // earlier may still hold their addresses, so they are freed only when
    // the matrix is freed.
    std::vector<void*> retired;
    b2sr_matrix* transpose = nullptr;
};

namespace b2sr {

// ---- status / allocation helpers (b2sr_api.cu) --------------------------------
void set_cuda_error(cudaError_t e);
void* dev_alloc(size_t bytes);
void dev_free(void* p);
void set_launch_count(int n);
void add_launch_count(int n);
// Kernel timer: records an event on `s` before (begin = true) or after the
// dominant kernel of a multiply while b2sr_kernel_timer_start armed it.
void kernel_timer_mark(cudaStream_t s, bool begin);

#define B2SR_CUDA_TRY(expr)                                   \
    do {                                                      \
        cudaError_t _e = (expr);                              \
        if (_e != cudaSuccess) {                              \
            ::b2sr::set_cuda_error(_e);                       \
            return B2SR_ERR_CUDA;                             \
        }                                                     \
    } while (0)

#define B2SR_LAUNCH_CHECK()                                   \
    do {                                                      \
        cudaError_t _e = cudaGetLastError();                  \
        if (_e != cudaSuccess) {                              \
            ::b2sr::set_cuda_error(_e);                       \
            return B2SR_ERR_CUDA;                             \
        }                                                     \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Launch `kernel` behind the previous kernel on `s` with programmatic
// dependent launch: its blocks may be scheduled while that grid drains and
// wait in griddep_wait() until it has completed and its writes are visible.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent(void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t s,
                                    Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// ---- packing (b2sr_pack.cu) ---------------------------------------------------
// Device CSR validation; writes error bits into *d_flag (0 = valid).
b2sr_status launch_validate_csr(const int* rowptr, const int* colind, int nrows, int ncols,
                                int nnz, int* d_flag, cudaStream_t s);
// Tiles per tile-row into d_counts[nb]; does nothing if *d_csr_flag != 0.
b2sr_status launch_count_tiles(const int* rowptr, const int* colind, int nrows, int nb, int T,
                               const int* d_csr_flag, int* d_counts, cudaStream_t s);
// In-place exclusive scan of d_vals[0..n) with the total written to d_vals[n].
// d_vals must have n + 1 entries.  d_err receives 1 if the total overflows int32.
b2sr_status launch_exclusive_scan(int* d_vals, int n, int* d_err, cudaStream_t s);
// Fill colind/tiles from CSR given the B2SR rowptr.
b2sr_status launch_fill_tiles(const int* rowptr, const int* colind, int nrows, int nb, int T,
                              const int* browptr, int* bcolind, void* tiles, cudaStream_t s);
b2sr_status launch_pack_vec_bits(const float* x, int n, int T, void* bits, cudaStream_t s);
b2sr_status launch_unpack_vec_bits(const void* bits, int n, int T, float* out, cudaStream_t s);
// Set bits of a B2SR matrix (for the descriptor); result in *d_count (int64).
b2sr_status launch_count_bits(const void* tiles, long long nwords, int T,
                              unsigned long long* d_count, cudaStream_t s);

// ---- transpose (b2sr_transpose.cu) ---------------------------------------------
// A^T's rowptr (nbc + 1 entries), colind and tiles (nt each) from A's, on the
// device (stable radix sort of the tiles by tile-column, then a bit transpose
// of every tile).  Synchronizes `s`.  B2SR_ERR_INVALID_VALUE if a tile-column
// lies outside [0, nbc).
b2sr_status launch_transpose(const int* rowptr, const int* colind, const void* tiles, int nb, int nbc, int nt, int T,
                             int* rowptr_t, int* colind_t, void* tiles_t, cudaStream_t s);

// ---- multiply (b2sr_spmv.cu) --------------------------------------------------
struct MatView {
    const int* rowptr;
    const int* colind;
    const void* tiles;
    int nb;
    int ncols;  // x length for bin_full_full (segments past it are read element-wise)
    int T;
};

// Merge-path start coordinates of `grid` equal shares of the nb + nt items.
// nt is read from rowptr[nb] on the device.
b2sr_status launch_partition(const MatView& A, int grid, Coord* d_starts, cudaStream_t s);

// Largest grid the merge-path multiply of (variant, T, shape) uses on this device.
int merge_grid(b2sr_variant v, int T, const LaunchShape& shape, int num_sms);
// Bytes of scratch the merge-path multiply needs for `grid` CTAs.
size_t carry_bytes(b2sr_variant v, int T, int grid);

// One multiply: main merge-path kernel + carry fix-up.  `carries` is scratch of
// carry_bytes(v, T, grid) bytes.  `mask` is used by the masked variant only.
b2sr_status launch_spmv(b2sr_variant v, const MatView& A, const LaunchShape& shape, int grid,
                        const Coord* d_starts, const void* x, void* y, const void* mask,
                        int accumulate, void* carries, cudaStream_t s);

// ---- dense right-hand sides (b2sr_spmm.cu) ---------------------------------------
constexpr int SPMM_CHUNK_ITEMS = 1024;
template <typename V>
b2sr_status spmm_launch(const MatView& A, const V* X, long long ldx, V* Y, long long ldy, int k,
                        int accumulate, const Coord* starts, int nchunks, void* scratch, int grid_warps,
                        cudaStream_t s);
size_t spmm_scratch_bytes(int T, int elem_bytes, int nchunks, int k);
int spmm_grid_warps(int num_sms);

// ---- row-task dense right-hand sides (b2sr_spmm_rows.cu) --------------------------
// Synchronizes `s` (it reads rowptr, and at T = 16 / 32 each tile-row's set
// bits, on the host).
b2sr_status spmm_rows_plan_create(const int* d_rowptr, const void* d_tiles, int nb, int T, int num_sms,
                                  SpmmRowsPlan* out, cudaStream_t s);
void spmm_rows_plan_free(SpmmRowsPlan* p);
size_t spmm_rows_scratch_bytes(const SpmmRowsPlan& p, int T, int elem_bytes, int k);
size_t spmm_rows_state_bytes(const SpmmRowsPlan& p);
template <typename V>
b2sr_status spmm_rows_launch(const MatView& A, const SpmmRowsPlan& p, const V* X, long long ldx, V* Y,
                             long long ldy, int k, int rhs_block, int accumulate, void* scratch, int* state,
                             int num_sms, cudaStream_t s);

// ---- row-binned bin_full_full (b2sr_rowbin.cu) ------------------------------------
// bits: the plan of the bit-vector kernels (longer long-row tasks at T = 4).
b2sr_status rowbin_plan_create(const int* d_rowptr, int nb, int T, bool bits, RowBinPlan* out, cudaStream_t s);
void rowbin_plan_free(RowBinPlan* p);
size_t rowbin_scratch_bytes(const RowBinPlan& p, int T, int value_bytes);
// Bit-vector variants on the same plan: kind 0 bin_bin_bin, 1 masked, 2 int32
// counts, 3 FP32 counts (bin_bin_full).
size_t rowbin_bits_scratch_bytes(const RowBinPlan& p, int T);
// The push side of an auto-direction product (b2sr_push.cu) as the pull
// kernels see it: they return at once when the push took the product.
struct PushLink {
    const int* ctl = nullptr;  // launch_push's counters; null: pull only
    long long nt = 0;
    int pct = 0;  // push when the active tiles are below pct% of nt
    bool gate = false;  // launch the pull from the device, only when chosen (not in a capture)
};
// timed: kernel timer marks around the main kernel.
b2sr_status rowbin_bits(const RowBinPlan& p, const MatView& A, int kind, const void* x, void* y, const void* mask,
                        int accumulate, void* partials, const PushLink& link, bool timed, cudaStream_t s);
// sparse_cols: load x only for each tile's set columns (launch option gather = 3,
// the default at T >= 16) instead of the tile-column's whole x segment.
b2sr_status rowbin_spmv(const RowBinPlan& p, const MatView& A, const float* x, float* y, int accumulate,
                        void* scratch, cudaTextureObject_t xtex, bool sparse_cols, cudaStream_t s);
b2sr_status rowbin_multi_bits(const RowBinPlan& p, const MatView& A, const void* x, void* y, const void* mask,
                              int word_bits, int accumulate, void* scratch, cudaTextureObject_t xtex,
                              cudaStream_t s);
// ---- direction-optimised bit-vector products (b2sr_push.cu) -------------------------
// The push form visits only the tile-columns whose x word is non-zero, through
// the transpose At; ctl[1] counts their tiles on the device.  Auto mode takes
// it below push_percent(T)% of nt: the tile share at which the push kernel and
// the row-binned pull kernel take equal time on R-MAT scale 20 (GB300; push
// time is close to linear in that share).
inline int push_percent(int T) { return T == 4 ? 18 : T == 8 ? 27 : T == 16 ? 45 : 85; }
__device__ __forceinline__ bool push_chosen(const int* ctl, int mode, long long nt, int pct) {
    return mode == 2 || (long long)ctl[1] * 100 < nt * pct;
}
// Scratch bytes of launch_push: counters and the work list.
size_t push_scratch_bytes(int nbc, long long nt);
// mode 1 (auto) or 2 (always push); kind as rowbin_bits.  Zeroes y (y_bytes)
// first unless accumulate.  Fills *link (counters, threshold) for the pull kernels
// launched after it.
b2sr_status launch_push(const MatView& At, int kind, int mode, const void* x, void* y, const void* mask,
                        int accumulate, size_t y_bytes, long long nt, void* scratch, int num_sms,
                        PushLink* link, int* hint, cudaStream_t s);
// Auto direction: the active-tile count of x alone (no work list, y untouched)
// into state[1] (state: 3 ints, zeroed, left zeroed), and from the last block
// the direction (1 push, 2 pull) into *hint.
b2sr_status launch_direction_count(const MatView& At, const void* x, long long nt, int* state, int* hint,
                                   cudaStream_t s);

// Cached texture object (uint4 texels) over [ptr, ptr + bytes), or 0 when the
// buffer cannot back one (alignment, size).
cudaTextureObject_t vector_texture(const void* ptr, size_t bytes);

}  // namespace b2sr
