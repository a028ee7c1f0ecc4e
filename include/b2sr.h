/*
 * b2sr.h — C ABI of the GB300 (sm_103a) B2SR binary SpMV library.
 *
 * B2SR ("bit-packed block sparse row") stores a 0/1 matrix as T x T tiles,
 * T in {4, 8, 16, 32}:
 *   rowptr[nb + 1]  int32   tiles of tile-row i are [rowptr[i], rowptr[i+1])
 *   colind[nt]      int32   tile-column of each tile, ascending within a tile-row
 *   tiles[nt * T]   words   word r of tile t holds row r of the tile; bit (T-1-c)
 *                           is column c (MSB = column 0).  Word type: uint8 for
 *                           T = 4 (low nibble used) and T = 8, uint16 for T = 16,
 *                           uint32 for T = 32.
 * nb = ceil(nrows / T) tile-rows, nbc = ceil(ncols / T) tile-columns.
 * This is the layout the reference builds with cusparseXcsr2bsrNnz +
 * cusparseScsr2bsr (CUSPARSE_DIRECTION_ROW) + ToBit{T}Col
 * (bmv_eval/backend/csr2bsr_batch_bsrbmv.cu:16-133, bmv_eval/backend/bsrbmv.cu:33-203),
 * so buffers are interchangeable with the reference kernels.
 *
 * Bit vectors ("bits" below) hold one word per T-block of a dense vector with
 * the same word type and bit order: bit (T-1-c) of word j is element j*T + c
 * (bmv_eval/backend/bsrbmv.cu:64-222, ToBit{T}Row).
 *
 * Conventions of every entry point:
 *   - pointers named d_* are device pointers; h_* are host pointers;
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream);
 *   - every call is stream-ordered and asynchronous unless stated otherwise;
 *   - dense outputs are padded like the reference's buffers: a float output of
 *     a matrix with nb tile-rows has nb*T entries, a bit output nb words;
 *   - `accumulate` != 0 means y += A.x (the reference kernels' behaviour,
 *     bsrbmv.cu:307,675,1079); 0 means y = A.x (no pre-zeroing needed);
 *   - argument errors are reported as a status before anything is launched.
 */
#ifndef B2SR_H_
#define B2SR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    B2SR_SUCCESS = 0,
    B2SR_ERR_INVALID_VALUE = 1,   /* null pointer, bad tile size, bad size */
    B2SR_ERR_INVALID_CSR = 2,     /* rowptr not monotone, colind out of range or unsorted */
    B2SR_ERR_ALLOC = 3,           /* device allocation failed */
    B2SR_ERR_CUDA = 4,            /* a CUDA runtime call failed */
    B2SR_ERR_NOT_SUPPORTED = 5,   /* combination not implemented */
    B2SR_ERR_OVERFLOW = 6,        /* sizes exceed the int32 index range */
    B2SR_ERR_DEVICE_CHECK = 7,    /* a device-side check reported an error */
    B2SR_ERR_IO = 8               /* packed-matrix file missing, short, or failing its checks */
} b2sr_status;

/* Multiply variants (names follow the reference kernels bmv{T}_{variant}). */
typedef enum {
    B2SR_BIN_BIN_BIN = 0,   /* bits x  -> bits y   (Boolean OR.AND)        bsrbmv.cu:277-613 */
    B2SR_BIN_BIN_FULL = 1,  /* bits x  -> float y  (neighbour counts)      bsrbmv.cu:618-821 */
    B2SR_BIN_FULL_FULL = 2, /* float x -> float y  (FP32 sum of set bits)  bsrbmv.cu:826-1081 */
    B2SR_BIN_BIN_COUNT = 3  /* bits x  -> int32 y  (exact neighbour counts; no reference kernel) */
} b2sr_variant;

/* Opaque matrix handle: device rowptr/colind/tiles plus cached launch data.
 * Immutable after packing; it may be shared between host threads.  Calls that
 * use the same handle on different streams may run concurrently. */
typedef struct b2sr_matrix b2sr_matrix;

typedef struct {
    int nrows, ncols;       /* scalar matrix shape */
    int tile_dim;           /* T */
    int nblockrows;         /* nb  = ceil(nrows / T) */
    int nblockcols;         /* nbc = ceil(ncols / T) */
    int nblocks;            /* nt, number of non-empty tiles */
    long long nnz;          /* set bits (= CSR nnz after de-duplication) */
    const int* d_rowptr;    /* device, nb + 1 */
    const int* d_colind;    /* device, nt */
    const void* d_tiles;    /* device, nt * T words */
    int owns_storage;       /* 1 if freed by b2sr_free */
} b2sr_matrix_desc;

/* ---- errors and version --------------------------------------------------- */
const char* b2sr_status_string(b2sr_status s);
/* Last CUDA error seen by the library on this host thread (cudaError_t as int). */
int b2sr_last_cuda_error(void);
int b2sr_version(void);  /* major*10000 + minor*100 + patch */

/* Allocation hook: every device allocation the library makes goes through it
 * (NULL restores cudaMalloc/cudaFree).  Lets a caller route allocations into
 * its own pool and lets tests inject allocation failures. */
typedef void* (*b2sr_alloc_fn)(size_t bytes, void* ctx);
typedef void (*b2sr_free_fn)(void* ptr, void* ctx);
void b2sr_set_allocator(b2sr_alloc_fn alloc_fn, b2sr_free_fn free_fn, void* ctx);

/* ---- packing -------------------------------------------------------------- */
/* CSR (int32, zero-based, column indices non-decreasing within each row;
 * duplicates allowed and merged) -> B2SR with tile size T, on the device.
 * Replaces CSR2HSBSF (bmv_eval/test_bin_full_full.cu:167-211) = cusparseXcsr2bsrNnz
 * + csr2bsr_batch_{T} (bmv_eval/backend/csr2bsr_batch_bsrbmv.cu:16,140,263,386).
 * The CSR is validated on the device first; a bad CSR returns
 * B2SR_ERR_INVALID_CSR and packs nothing.  Synchronises `stream` once (the tile
 * count decides the allocation size). */
b2sr_status b2sr_pack_csr(const int* d_rowptr, const int* d_colind, int nrows, int ncols,
                          int nnz, int tile_dim, void* stream, b2sr_matrix** out);

/* Wrap caller-owned B2SR arrays (for example ones built by the reference
 * packer).  Nothing is copied; the arrays must outlive the handle.  nblocks
 * must equal d_rowptr[nblockrows]. */
b2sr_status b2sr_matrix_wrap(const int* d_rowptr, const int* d_colind, const void* d_tiles,
                             int nrows, int ncols, int nblocks, int tile_dim, void* stream,
                             b2sr_matrix** out);

/* B2SR of the transpose, built once on the device and cached inside `m`
 * (used by the adjoint and the push direction).  Returns the cached handle,
 * owned by `m`.  The first call synchronizes `stream`; inside a stream
 * capture it returns B2SR_ERR_NOT_SUPPORTED unless the transpose exists.
 * B2SR_ERR_INVALID_VALUE: a tile-column of `m` outside the matrix. */
b2sr_status b2sr_matrix_transpose(b2sr_matrix* m, void* stream, const b2sr_matrix** out_t);

b2sr_status b2sr_matrix_describe(const b2sr_matrix* m, b2sr_matrix_desc* out);
void b2sr_free(b2sr_matrix* m);

/* Copy the B2SR arrays to host buffers sized from b2sr_matrix_describe
 * (rowptr nb+1 ints, colind nt ints, tiles nt*T words).  Synchronous. */
b2sr_status b2sr_matrix_download(const b2sr_matrix* m, int* h_rowptr, int* h_colind,
                                 void* h_tiles);

/* ---- packed B2SR files ------------------------------------------------------ */
/* A packed matrix on disk, so a later run skips CSR -> B2SR packing.  The file
 * is a 64-byte little-endian header -- magic "B2SRPACK", format version 1,
 * tile_dim, nrows, ncols, nblockrows, nblocks, nnz, and an FNV-1a 64-bit
 * checksum of the payload -- followed by rowptr (nblockrows + 1 int32), colind
 * (nblocks int32) and tiles (nblocks * T words).  The reference names such a
 * cache for its CSR (bmv_eval/backend/readMtx.hpp:229-246, 389-406) but never
 * writes it.  Both calls are synchronous.  b2sr_matrix_load checks the header,
 * the checksum and the structure (rowptr monotone and ending at nblocks,
 * colind in range and ascending within each tile-row) and returns B2SR_ERR_IO
 * when any check fails. */
b2sr_status b2sr_matrix_save(const b2sr_matrix* m, const char* path);
b2sr_status b2sr_matrix_load(const char* path, void* stream, b2sr_matrix** out);

/* ---- dense vector <-> bit vector ------------------------------------------ */
/* bits[j] word = (x[j*T + c] > 0) at bit (T-1-c), c < T; elements at or past n
 * give 0.  Writes ceil(n / T) words.  Replaces ToBit{T}Row
 * (bmv_eval/backend/bsrbmv.cu:64-222) + packRandVec (bmv_eval/test_bin_bin_bin.cu:249-282). */
b2sr_status b2sr_pack_vec_bits(const float* d_x, int n, int tile_dim, void* d_bits, void* stream);
/* out[i] = bit i as 0.0f / 1.0f for i < n.  Replaces bin2full
 * (bmv_eval/backend/utility.cu:156-178). */
b2sr_status b2sr_unpack_vec_bits(const void* d_bits, int n, int tile_dim, float* d_out,
                                 void* stream);

/* ---- multiply: single vector ---------------------------------------------- */
/* y = A.x over the Boolean semiring; x: nbc words, y: nb words.
 * Replaces bmv{4,8,16,32}_bin_bin_bin (bmv_eval/backend/bsrbmv.cu:277,437,508,579). */
b2sr_status b2sr_spmv_bin_bin_bin(const b2sr_matrix* m, const void* d_xbits, void* d_ybits,
                                  int accumulate, void* stream);
/* y[i] = number of j with A[i][j] = 1 and x_j = 1, stored as float (exact below
 * 2^24); x: nbc words, y: nb*T floats.
 * Replaces bmv{4,8,16,32}_bin_bin_full (bmv_eval/backend/bsrbmv.cu:618,678,738,789). */
b2sr_status b2sr_spmv_bin_bin_full(const b2sr_matrix* m, const void* d_xbits, float* d_y,
                                   int accumulate, void* stream);
/* Same counts as int32 (no reference counterpart; the int32-count workload). */
b2sr_status b2sr_spmv_bin_bin_count(const b2sr_matrix* m, const void* d_xbits, int* d_y,
                                    int accumulate, void* stream);
/* y = A.x in FP32, deterministic (fixed summation order, no float atomics);
 * x: at least ncols floats, y: nb*T floats, both 16-byte aligned.
 * Replaces bmv{4,8,16,32}_bin_full_full (bmv_eval/backend/bsrbmv.cu:826,899,975,1040). */
b2sr_status b2sr_spmv_bin_full_full(const b2sr_matrix* m, const float* d_x, float* d_y,
                                    int accumulate, void* stream);

/* Masked BFS step: y = (A.x) AND NOT mask, overwriting y; mask and y: nb words.
 * Replaces bmv{4,8,16,32}_bin_bin_bin_masked (bmv_eval/backend/bsrbmv.cu:1086-1229),
 * with the T = 8/16 shift defects of that code (bsrbmv.cu:1153,1189) not reproduced. */
b2sr_status b2sr_spmv_bin_bin_bin_masked(const b2sr_matrix* m, const void* d_xbits,
                                         const void* d_maskbits, void* d_ybits, void* stream);

/* ---- multiply: many frontiers at once ------------------------------------- */
/* Multi-source Boolean step: word_bits (32 or 64) frontiers packed one bit
 * each into a word per vertex; y[v] = OR of x[u] over the neighbours u of v
 * (row v of A), i.e. all frontiers advance in one pass.  x: ncols words,
 * y: nb*T words (uint32 or uint64), both 16-byte aligned.  With d_mask
 * (nb*T words, e.g. the visited sets) y = result AND NOT mask (accumulate
 * must then be 0); accumulate != 0 ORs into y.  No reference counterpart:
 * the reference advances one frontier per launch (bmv{T}_bin_bin_bin,
 * bmv_eval/backend/bsrbmv.cu:277-613). */
b2sr_status b2sr_spmv_multi_bits(const b2sr_matrix* m, const void* d_x, void* d_y, int word_bits,
                                 const void* d_mask, int accumulate, void* stream);

/* ---- multiply: dense right-hand sides (feature blocks) -------------------- */
/* Y = A . X (accumulate: Y += A . X) with X [ncols, k] and Y [nb*T, k]
 * row-major, row strides ldx >= k and ldy >= k (elements).  Deterministic:
 * each output is summed in a fixed order.  The adjoint dX = A^T . dY is this
 * call on b2sr_matrix_transpose(m).  No reference counterpart: the reference
 * multiplies one vector per launch (bmv_eval/backend/bsrbmv.cu:826-1081); this
 * is the multi-RHS form of its bin_full_full. */
b2sr_status b2sr_spmm_bin_full_full(const b2sr_matrix* m, const float* d_X, int k, long long ldx,
                                    float* d_Y, long long ldy, int accumulate, void* stream);
/* The same in FP64 (used for finite-difference gradient checks). */
b2sr_status b2sr_spmm_bin_full_full_f64(const b2sr_matrix* m, const double* d_X, int k, long long ldx,
                                        double* d_Y, long long ldy, int accumulate, void* stream);

/* ---- launch-shape control (autotuner hooks) ------------------------------- */
typedef struct {
    int threads;          /* merge path: threads per CTA, 128 or 256 (0 = default) */
    int items_per_thread; /* merge path: items per thread, 4 or 8 (and 16 with 128 threads) */
    int ctas_per_sm;      /* merge path: persistent CTAs per SM (0 = occupancy maximum) */
    int algorithm;        /* 0 = default (row-binned for every variant), 1 = merge path,
                             2 = row-binned */
    int gather;           /* row-binned x gathers (bin_full_full and multi-frontier): 0 = default,
                             1 = ld.global, 2 = texture fetches (x 512-byte aligned), 3 = only the
                             x elements of each tile's set columns (bin_full_full; the default at
                             T = 16 and 32, texture fetches at T = 4 and 8) */
    int rhs_block;        /* dense-RHS product (bin_full_full, T = 4/8): columns per warp pass,
                             16, 32, 64 or 128 for FP32 (half for FP64); 0 = the narrowest block
                             that covers k.  Narrower blocks load more X rows per warp instruction. */
    int direction;        /* bit-vector variants (row-binned): 0 = pull over every tile-row (default),
                             1 = auto: push through b2sr_matrix_transpose(m) when the tile-columns
                             with a non-zero x word hold under 18% (T = 4), 27% (8), 45% (16) or
                             85% (32) of the tiles, chosen on the device per call; 2 = always push.  The transpose is built on the first
                             such call (synchronizing), so make one before capturing a graph: during
                             capture without it, auto pulls and push returns B2SR_ERR_NOT_SUPPORTED.
                             Results equal the pull's bit for bit; bin_bin_full with accumulate or
                             more than 2^24 columns always pulls.  With T < 32 the push ORs into y
                             through 32-bit atomics on the aligned words holding y's words, so the
                             up to 3 bytes sharing a word with y's first or last word are read
                             and rewritten unchanged. */
} b2sr_launch_config;
/* Set the launch shape that later multiplies on `m` use (per variant). */
b2sr_status b2sr_matrix_set_launch(b2sr_matrix* m, b2sr_variant v, const b2sr_launch_config* cfg);
b2sr_status b2sr_matrix_get_launch(const b2sr_matrix* m, b2sr_variant v, b2sr_launch_config* cfg);

/* ---- autotuner -------------------------------------------------------------- */
typedef struct {
    int tile_dim;          /* chosen T */
    int algorithm;         /* chosen b2sr_launch_config.algorithm */
    int gather;            /* chosen b2sr_launch_config.gather */
    int threads;           /* merge-path shape (0 when not the merge path) */
    int items_per_thread;
    float best_ms;         /* median time of the chosen configuration */
    int candidates;        /* configurations timed (0 = taken from the cache) */
    int rhs_block;         /* chosen b2sr_launch_config.rhs_block (dense-RHS products) */
} b2sr_tune_result;

/* Packs the CSR at each tile size in tile_dims (NULL: 4, 8, 16, 32), times
 * the multiply of kind `variant` (k = 0: single vector; k > 0: the dense-RHS
 * product with k columns, bin_full_full only) under each launch option on
 * this device, and returns in *out the fastest packed matrix with that option
 * applied.  Decisions are cached per (rows, cols, nnz, kind, k, SM count) for
 * the process and, if B2SR_TUNE_CACHE names a file, in that file.  Runs
 * synchronously.  No reference counterpart: the reference fixes T at compile
 * time (-DTILEDIM, bmv_eval/Makefile:11-44) and picks launch shapes by hand. */
b2sr_status b2sr_autotune(const int* d_rowptr, const int* d_colind, int nrows, int ncols, int nnz,
                          b2sr_variant variant, int k, const int* tile_dims, int n_tile_dims,
                          void* stream, b2sr_matrix** out, b2sr_tune_result* result);
void b2sr_autotune_clear_cache(void);

/* Number of kernels the last multiply call on this host thread launched. */
int b2sr_last_launch_count(void);

/* Kernel timer (a measurement aid for benchmarks and profiling).  While armed,
 * each multiply call records a CUDA event pair on its launching stream around
 * its dominant kernel (the row-binned, merge-path or dense-RHS kernel, not the
 * carry fix-up), for the first `capacity` calls; calls made during stream
 * capture are not recorded.  b2sr_kernel_timer_read waits for the recorded
 * events, writes up to `capacity` durations in milliseconds, disarms the timer
 * and returns how many it wrote (or -1 on a CUDA error). */
b2sr_status b2sr_kernel_timer_start(int capacity);
int b2sr_kernel_timer_read(float* ms, int capacity);

/* ---- reference-compatible shims ------------------------------------------- */
/* Same signatures and host-side semantics as the reference, so its test_bin_*
 * drivers relink against this library with only their launch lines changed.
 * Default stream; `accumulate` behaviour as the reference kernels (+= and |=). */

/* cusparseXcsr2bsrNnz replacement (bmv_eval/test_bin_full_full.cu:189-190):
 * fills d_bsrRowPtr (nb + 1) and returns the tile count in *h_nblocks. */
b2sr_status b2sr_ref_csr2bsr_nnz(const int* d_csrRowPtr, const int* d_csrColInd, int nrows,
                                 int ncols, int blocksize, int* d_bsrRowPtr, int* h_nblocks);
/* csr2bsr_batch_{4,8,16,32} replacement (bmv_eval/backend/csr2bsr_batch_bsrbmv.cu:16-19,
 * 140-143, 263-266, 386-389): host CSR in, device B2SR out; d_bsrRowPtr must
 * already hold the structure from b2sr_ref_csr2bsr_nnz.  Unlike the reference
 * it copies all nblocks*blocksize words for T = 16/32. */
b2sr_status b2sr_ref_csr2bsr_batch(const int* h_csrRowPtr, const int* h_csrColInd, int nrows,
                                   int ncols, int nnz, int* d_bsrRowPtr, int* d_bsrColInd,
                                   void* d_bsrVal, int blocksize, int nblockrows, int nblocks);
/* Kernel-launch replacements with the reference kernel signatures
 * (A tiles, B = x, C = y, rowptr, colind, nblockrows), accumulating
 * (+= and |=) on the legacy default stream; each replaces the launch of
 * bmv{T}_{variant} in the drivers' timed loops
 * (bmv_eval/test_bin_full_full.cu:285-297, test_bin_bin_bin.cu:358-369,
 * test_bin_bin_full.cu:311-353).  The matrix is square with nblockrows*T
 * rows; x holds nblockrows*T floats (16-byte aligned, as y) or nblockrows
 * words.  The first call on a set of arrays reads the tile count from
 * rowptr[nblockrows] (synchronizing) and builds the row-binned plan; the
 * library caches both per (device, rowptr, colind, A, nblockrows, tile_dim),
 * so later calls launch the same kernels as the matrix API with no
 * allocation and no synchronization.  The arrays must therefore not change
 * while they are cached: b2sr_ref_csr2bsr_nnz and b2sr_ref_csr2bsr_batch drop
 * the entries of the arrays they write, and b2sr_ref_release drops others. */
b2sr_status b2sr_ref_bmv_bin_bin_bin(int tile_dim, const void* A, const void* B, void* C,
                                     const int* rowptr, const int* colind, int nblockrows);
b2sr_status b2sr_ref_bmv_bin_bin_full(int tile_dim, const void* A, const void* B, float* C,
                                      const int* rowptr, const int* colind, int nblockrows);
b2sr_status b2sr_ref_bmv_bin_full_full(int tile_dim, const void* A, const float* B, float* C,
                                       const int* rowptr, const int* colind, int nblockrows);
/* Drops the shims' cached plan of the arrays whose rowptr is `rowptr` (NULL:
 * every cached plan), synchronizing the device first if anything is dropped.
 * Call it before freeing or rewriting arrays passed to the shims above other
 * than through the packer shims.  No reference counterpart (the reference
 * has no state between launches). */
void b2sr_ref_release(const int* rowptr);

/* ---- allocation-free multiply ---------------------------------------------- */
/* y = A.x (accumulate: y += A.x) in FP32 on raw B2SR arrays, like
 * b2sr_ref_bmv_bin_full_full but on `stream`, with ncols bounding the x reads,
 * and without allocating anything: for callers that cannot allocate device
 * memory while they multiply (a fully reserved memory budget, real-time loops
 * where cudaMalloc/cudaFree would stall or synchronize the device, hosts that
 * forbid the CUDA allocator).  Its scratch is a fixed 192 KB array in device
 * memory that the library holds on every GPU that loads it.  The first call
 * on each device looks that array's address up (cudaGetSymbolAddress) and
 * should come before any stream capture.  All calls share the array: calls
 * whose GPU work overlaps race.  Returns B2SR_ERR_NOT_SUPPORTED when the
 * device needs more scratch than the array holds (more than ~1200 CTAs).
 * x and y 16-byte aligned.  No counterpart in the reference. */
b2sr_status b2sr_spmv_bin_full_full_noalloc(int tile_dim, const void* d_tiles, const int* d_rowptr,
                                            const int* d_colind, int nblockrows, int ncols,
                                            const float* d_x, float* d_y, int accumulate, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* B2SR_H_ */
