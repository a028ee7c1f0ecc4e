// CSR -> B2SR packing on the device, and dense <-> bit vector conversion.
//
// The reference packs on the host, one tile-row at a time: per non-empty
// tile-row it copies a CSR slab to the device, expands it to dense float tiles
// with cusparseScsr2bsr and bit-packs them with ToBit{T}Col
// (bmv_eval/backend/csr2bsr_batch_bsrbmv.cu:34-133, bmv_eval/backend/bsrbmv.cu:33-203).
// Here the whole matrix is packed by three device passes with no float
// expansion: count tiles per tile-row, exclusive scan, fill.  One warp serves
// 32/T tile-rows; lane r of a group walks CSR row r of its tile-row, and the
// group repeatedly takes the smallest pending tile-column (a T-way merge of the
// sorted rows), so tiles come out in ascending tile-column order, the order
// cusparseScsr2bsr produces.
#include "b2sr_common.cuh"

namespace b2sr {

enum : int { CSR_BAD_ROWPTR = 1, CSR_BAD_COLIND = 2, CSR_UNSORTED = 4 };

// rowptr[0] == 0, rowptr[nrows] == nnz, 0 <= rowptr[i] <= rowptr[i+1] <= nnz;
// colind in [0, ncols) and non-decreasing within each row.  One warp per row;
// reads are clamped so a broken rowptr cannot send them out of bounds.
__global__ void validate_csr_kernel(const int* __restrict__ rowptr, const int* __restrict__ colind,
                                    int nrows, int ncols, int nnz, int* __restrict__ flag) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    int bad = 0;
    if (warp == 0 && lane == 0) {
        if (rowptr[0] != 0 || rowptr[nrows] != nnz) bad |= CSR_BAD_ROWPTR;
    }
    for (long long row = warp; row < nrows; row += nwarps) {
        int b = rowptr[row], e = rowptr[row + 1];
        if (b < 0 || e < b || e > nnz) {
            bad |= CSR_BAD_ROWPTR;
            b = min(max(b, 0), nnz);
            e = min(max(e, b), nnz);
        }
        for (int p = b + lane; p < e; p += 32) {
            int c = colind[p];
            if (c < 0 || c >= ncols) bad |= CSR_BAD_COLIND;
            if (p > b && colind[p - 1] > c) bad |= CSR_UNSORTED;
        }
    }
    bad = __reduce_or_sync(FULL_MASK, bad);
    if (lane == 0 && bad) atomicOr(flag, bad);
}

b2sr_status launch_validate_csr(const int* rowptr, const int* colind, int nrows, int ncols,
                                int nnz, int* d_flag, cudaStream_t s) {
    B2SR_CUDA_TRY(cudaMemsetAsync(d_flag, 0, sizeof(int), s));
    const int threads = 256;
    long long warps = nrows > 0 ? nrows : 1;
    long long blocks = (warps * 32 + threads - 1) / threads;
    if (blocks > 65535LL * 16) blocks = 65535LL * 16;
    validate_csr_kernel<<<(unsigned)blocks, threads, 0, s>>>(rowptr, colind, nrows, ncols, nnz,
                                                            d_flag);
    B2SR_LAUNCH_CHECK();
    return B2SR_SUCCESS;
}

// Chunks: a tile-row whose longest CSR row (its lead row) has L entries is
// cut into ceil(L / PACK_CHUNK) chunks at the tile-columns of lead-row entries
// PACK_CHUNK, 2*PACK_CHUNK, ...; chunk k covers the tile-columns
// [lo_k, lo_{k+1}), so the chunks of a tile-row partition its tiles and emit
// them in tile-column order.  Hub tile-rows thus spread over many lane groups
// instead of one serial merge.
constexpr int PACK_CHUNK = 256;

__global__ void chunk_plan_kernel(const int* __restrict__ rowptr, int nrows, int nb, int T, int* __restrict__ nch) {
    const long long tr = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tr >= nb) return;
    int lead = 0;
    for (int r = 0; r < T; ++r) {
        const long long row = tr * T + r;
        if (row < nrows) lead = max(lead, rowptr[row + 1] - rowptr[row]);
    }
    nch[tr] = max(1, (lead + PACK_CHUNK - 1) / PACK_CHUNK);
}

// First index in [b, e) whose column is >= key (colind ascending in [b, e)).
__device__ __forceinline__ int lower_bound_col(const int* __restrict__ colind, int b, int e, long long key) {
    while (b < e) {
        const int m = b + ((e - b) >> 1);
        if ((long long)colind[m] < key) b = m + 1;
        else e = m;
    }
    return b;
}

// The T-way merge shared by the count and fill passes.  Each group of T lanes
// owns one chunk; lane r walks its part of CSR row tr*T + r.  Per step the
// group takes the smallest pending tile-column m, every lane ORs the bits of
// its entries in tile-column m into its row word, and the tile is emitted.
// The loop runs until every group of the warp is exhausted, so the shuffles
// see full warps.  choff: exclusive scan of the chunks per tile-row (nb + 1
// entries); count pass: ccount[c] = tiles of chunk c; fill pass: chunk c
// writes from browptr[tr] + coff[c] - coff[choff[tr]] on.
template <int T, bool FILL>
__global__ void __launch_bounds__(256)
merge_chunks_kernel(const int* __restrict__ rowptr, const int* __restrict__ colind, int nrows, int nb,
                    const int* __restrict__ choff, int nchunks, int* __restrict__ ccount,
                    const int* __restrict__ coff, const int* __restrict__ browptr, int* __restrict__ bcolind,
                    typename TileWord<T>::type* __restrict__ tiles) {
    using W = typename TileWord<T>::type;
    constexpr int G = 32 / T;
    constexpr int LT = Log2<T>::value;
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int g = lane / T, r = lane % T;
    const long long c = warp * G + g;
    if (__all_sync(FULL_MASK, c >= nchunks)) return;
    const bool live = c < nchunks;
    // tile-row of the chunk: the last tr with choff[tr] <= c (choff strictly increasing)
    int tr = 0;
    if (live) {
        int lo = 0, hi = nb;  // choff[lo] <= c < choff[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (choff[mid] <= c) lo = mid;
            else hi = mid;
        }
        tr = lo;
    }
    const int k = live ? (int)(c - choff[tr]) : 0, nk = live ? choff[tr + 1] - choff[tr] : 1;
    const long long row = (long long)tr * T + r;
    const bool valid = live && row < nrows;
    const int rs = valid ? rowptr[row] : 0, re = valid ? rowptr[row + 1] : 0;
    // lead row of the tile-row: longest, lowest r on ties
    int best_len = valid ? re - rs : -1, best_r = r, lead_rs = rs;
#pragma unroll
    for (int o = 1; o < T; o <<= 1) {
        const int ol = __shfl_xor_sync(FULL_MASK, best_len, o);
        const int orr = __shfl_xor_sync(FULL_MASK, best_r, o);
        const int ors = __shfl_xor_sync(FULL_MASK, lead_rs, o);
        if (ol > best_len || (ol == best_len && orr < best_r)) {
            best_len = ol;
            best_r = orr;
            lead_rs = ors;
        }
    }
    int p = rs, e = re;
    if (live && nk > 1) {
        if (k > 0) p = lower_bound_col(colind, rs, re, (long long)(colind[lead_rs + k * PACK_CHUNK] >> LT) << LT);
        if (k + 1 < nk) e = lower_bound_col(colind, rs, re, (long long)(colind[lead_rs + (k + 1) * PACK_CHUNK] >> LT) << LT);
    }
    int out = 0;
    if (FILL && live) out = browptr[tr] + coff[c] - coff[choff[tr]];
    int cnt = 0;
    while (true) {
        int m = (p < e) ? (colind[p] >> LT) : INT_MAX;
#pragma unroll
        for (int o = 1; o < T; o <<= 1) m = min(m, __shfl_xor_sync(FULL_MASK, m, o));
        if (__all_sync(FULL_MASK, m == INT_MAX)) break;
        if (m != INT_MAX) {
            uint32_t bits = 0;
            while (p < e) {
                const int col = colind[p];
                if ((col >> LT) != m) break;
                bits |= 1u << (T - 1 - (col & (T - 1)));
                ++p;
            }
            if (FILL) {
                tiles[(size_t)out * T + r] = (W)bits;
                if (r == 0) bcolind[out] = m;
                ++out;
            }
            ++cnt;
        }
    }
    if (!FILL && r == 0 && live) ccount[c] = cnt;
}

// counts[tr] = sum of the tiles of tile-row tr's chunks.
__global__ void chunk_sum_kernel(const int* __restrict__ choff, const int* __restrict__ ccount, int nb,
                                 int* __restrict__ counts) {
    const long long tr = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tr >= nb) return;
    int s = 0;
    for (int c = choff[tr]; c < choff[tr + 1]; ++c) s += ccount[c];
    counts[tr] = s;
}

template <int T, bool FILL>
static void launch_merge_chunks(const int* rowptr, const int* colind, int nrows, int nb, const int* choff,
                                int nchunks, int* ccount, const int* coff, const int* browptr, int* bcolind,
                                void* tiles, cudaStream_t s) {
    constexpr int G = 32 / T;
    const long long warps = ((long long)nchunks + G - 1) / G;
    const long long blocks = (warps * 32 + 255) / 256;
    if (blocks == 0) return;
    merge_chunks_kernel<T, FILL><<<(unsigned)blocks, 256, 0, s>>>(
        rowptr, colind, nrows, nb, choff, nchunks, ccount, coff, browptr, bcolind,
        reinterpret_cast<typename TileWord<T>::type*>(tiles));
}

static void merge_chunks(bool fill, int T, const int* rowptr, const int* colind, int nrows, int nb, const int* choff,
                         int nchunks, int* ccount, const int* coff, const int* browptr, int* bcolind, void* tiles,
                         cudaStream_t s) {
#define B2SR_MERGE_T(TT)                                                                                     \
    if (T == TT) {                                                                                           \
        if (fill) launch_merge_chunks<TT, true>(rowptr, colind, nrows, nb, choff, nchunks, ccount, coff,     \
                                                browptr, bcolind, tiles, s);                                 \
        else launch_merge_chunks<TT, false>(rowptr, colind, nrows, nb, choff, nchunks, ccount, coff,         \
                                            browptr, bcolind, tiles, s);                                     \
    }
    B2SR_MERGE_T(4) B2SR_MERGE_T(8) B2SR_MERGE_T(16) B2SR_MERGE_T(32)
#undef B2SR_MERGE_T
}

// The chunks of every tile-row: choff (nb + 1, exclusive scan) and their
// number.  Synchronises `s`.
static b2sr_status plan_chunks(const int* rowptr, int nrows, int nb, int T, int** d_choff, int* nchunks,
                               cudaStream_t s) {
    int* choff = static_cast<int*>(dev_alloc(sizeof(int) * ((size_t)nb + 2)));
    if (!choff) return B2SR_ERR_ALLOC;
    int* err = choff + nb + 1;
    if (nb > 0) {
        chunk_plan_kernel<<<(nb + 255) / 256, 256, 0, s>>>(rowptr, nrows, nb, T, choff);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_cuda_error(e);
            dev_free(choff);
            return B2SR_ERR_CUDA;
        }
    }
    b2sr_status st = launch_exclusive_scan(choff, nb, err, s);  // synchronises s
    int h[2] = {0, 0};
    if (st == B2SR_SUCCESS) {
        cudaError_t e = cudaMemcpy(h, choff + nb, 2 * sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            set_cuda_error(e);
            st = B2SR_ERR_CUDA;
        } else if (h[1] != 0) {
            st = B2SR_ERR_OVERFLOW;
        }
    }
    if (st != B2SR_SUCCESS) {
        dev_free(choff);
        return st;
    }
    *d_choff = choff;
    *nchunks = h[0];
    return B2SR_SUCCESS;
}

b2sr_status launch_count_tiles(const int* rowptr, const int* colind, int nrows, int nb, int T,
                               const int* d_csr_flag, int* d_counts, cudaStream_t s) {
    if (!valid_tile(T)) return B2SR_ERR_INVALID_VALUE;
    if (d_csr_flag) {  // an invalid CSR is reported by the caller; plan nothing on it
        int flag = 0;
        cudaError_t e = cudaMemcpyAsync(&flag, d_csr_flag, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_cuda_error(e);
            return B2SR_ERR_CUDA;
        }
        if (flag != 0) return B2SR_SUCCESS;
    }
    int* choff = nullptr;
    int nchunks = 0;
    b2sr_status st = plan_chunks(rowptr, nrows, nb, T, &choff, &nchunks, s);
    if (st != B2SR_SUCCESS) return st;
    int* ccount = static_cast<int*>(dev_alloc(sizeof(int) * ((size_t)nchunks + 1)));
    if (!ccount) {
        dev_free(choff);
        return B2SR_ERR_ALLOC;
    }
    merge_chunks(false, T, rowptr, colind, nrows, nb, choff, nchunks, ccount, nullptr, nullptr, nullptr, nullptr, s);
    if (nb > 0) chunk_sum_kernel<<<(nb + 255) / 256, 256, 0, s>>>(choff, ccount, nb, d_counts);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // scratch is freed below
    dev_free(ccount);
    dev_free(choff);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return B2SR_ERR_CUDA;
    }
    return B2SR_SUCCESS;
}

b2sr_status launch_fill_tiles(const int* rowptr, const int* colind, int nrows, int nb, int T,
                              const int* browptr, int* bcolind, void* tiles, cudaStream_t s) {
    if (!valid_tile(T)) return B2SR_ERR_INVALID_VALUE;
    int* choff = nullptr;
    int nchunks = 0;
    b2sr_status st = plan_chunks(rowptr, nrows, nb, T, &choff, &nchunks, s);
    if (st != B2SR_SUCCESS) return st;
    // chunk offsets: count the chunks again, exclusive scan
    int* coff = static_cast<int*>(dev_alloc(sizeof(int) * ((size_t)nchunks + 2)));
    if (!coff) {
        dev_free(choff);
        return B2SR_ERR_ALLOC;
    }
    merge_chunks(false, T, rowptr, colind, nrows, nb, choff, nchunks, coff, nullptr, nullptr, nullptr, nullptr, s);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        st = launch_exclusive_scan(coff, nchunks, coff + nchunks + 1, s);  // synchronises s
        if (st == B2SR_SUCCESS)
            merge_chunks(true, T, rowptr, colind, nrows, nb, choff, nchunks, nullptr, coff, browptr, bcolind, tiles,
                         s);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // scratch is freed below
    }
    dev_free(coff);
    dev_free(choff);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return B2SR_ERR_CUDA;
    }
    return st;
}

// ---- exclusive scan -------------------------------------------------------------
// Three kernels: per-block sums, a scan of the block sums in one CTA, and the
// per-block scan with the block offset.  Sums are kept in 64 bits so an int32
// overflow of the total is detected instead of wrapping.
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ long long block_sum_ll(long long v, long long* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL_MASK, v, o);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL_MASK, v, o);
    }
    __syncthreads();
    return v;  // valid in thread 0
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and stores the block total in *total.
__device__ __forceinline__ long long block_exscan_ll(long long v, long long* sh, long long* total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        long long u = __shfl_up_sync(FULL_MASK, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) sh[w] = inc;
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        long long s = lane < nw ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            long long u = __shfl_up_sync(FULL_MASK, s, o);
            if (lane >= o) s += u;
        }
        if (lane < nw) sh[lane] = s;  // inclusive warp totals
    }
    __syncthreads();
    const long long warp_off = w > 0 ? sh[w - 1] : 0;
    *total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_off + inc - v;
}

__global__ void __launch_bounds__(SCAN_THREADS)
scan_reduce_kernel(const int* __restrict__ vals, int n, long long* __restrict__ partial) {
    __shared__ long long sh[32];
    const long long base = (long long)blockIdx.x * SCAN_TILE;
    long long v = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        long long i = base + (long long)k * SCAN_THREADS + threadIdx.x;
        if (i < n) v += vals[i];
    }
    v = block_sum_ll(v, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
}

__global__ void __launch_bounds__(SCAN_THREADS)
scan_partials_kernel(long long* __restrict__ partial, int nblocks) {
    __shared__ long long sh[32];
    long long carry = 0;
    for (int base = 0; base < nblocks; base += SCAN_THREADS) {
        const int i = base + threadIdx.x;
        long long v = i < nblocks ? partial[i] : 0;
        long long total;
        long long ex = block_exscan_ll(v, sh, &total);
        if (i < nblocks) partial[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) partial[nblocks] = carry;
}

__global__ void __launch_bounds__(SCAN_THREADS)
scan_apply_kernel(int* __restrict__ vals, int n, const long long* __restrict__ partial,
                  int nblocks, int* __restrict__ err) {
    __shared__ long long sh[32];
    const long long base = (long long)blockIdx.x * SCAN_TILE;
    // Each thread owns SCAN_ITEMS consecutive elements.
    const long long first = base + (long long)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    long long local = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = (first + k < n) ? vals[first + k] : 0;
        local += v[k];
    }
    long long total;
    long long ex = block_exscan_ll(local, sh, &total) + partial[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (first + k < n) {
            if (ex > INT_MAX) *err = 1;
            vals[first + k] = (int)ex;
        }
        ex += v[k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const long long all = partial[nblocks];
        if (all > INT_MAX) *err = 1;
        vals[n] = (int)(all > INT_MAX ? INT_MAX : all);
    }
}

b2sr_status launch_exclusive_scan(int* d_vals, int n, int* d_err, cudaStream_t s) {
    B2SR_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), s));
    const int nblocks = n > 0 ? (n + SCAN_TILE - 1) / SCAN_TILE : 1;
    long long* partial = static_cast<long long*>(dev_alloc(sizeof(long long) * (nblocks + 1)));
    if (!partial) return B2SR_ERR_ALLOC;
    scan_reduce_kernel<<<nblocks, SCAN_THREADS, 0, s>>>(d_vals, n, partial);
    scan_partials_kernel<<<1, SCAN_THREADS, 0, s>>>(partial, nblocks);
    scan_apply_kernel<<<nblocks, SCAN_THREADS, 0, s>>>(d_vals, n, partial, nblocks, d_err);
    cudaError_t e = cudaGetLastError();
    // The scratch is freed after the stream drains: the caller synchronises the
    // stream right after the scan (it needs the total on the host).
    cudaError_t e2 = cudaStreamSynchronize(s);
    dev_free(partial);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        set_cuda_error(e != cudaSuccess ? e : e2);
        return B2SR_ERR_CUDA;
    }
    return B2SR_SUCCESS;
}

// ---- dense <-> bits ---------------------------------------------------------------
// A warp votes on 32 consecutive elements; the bit-reversed ballot holds
// element 32k + l at bit 31 - l, i.e. 32/T words of the MSB-first layout side
// by side (ToBit{T}Row order, bmv_eval/backend/bsrbmv.cu:64-222).
template <int T>
__global__ void pack_vec_bits_kernel(const float* __restrict__ x, long long n,
                                     typename TileWord<T>::type* __restrict__ bits,
                                     long long nwords) {
    using W = typename TileWord<T>::type;
    constexpr int PER = 32 / T;  // words per ballot
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long chunk = warp; chunk * 32 < n; chunk += nwarps) {
        const long long i = chunk * 32 + lane;
        const bool v = i < n && x[i] > 0.0f;
        const uint32_t word32 = __brev(__ballot_sync(FULL_MASK, v));
        if (lane < PER) {
            const long long wi = chunk * PER + lane;
            if (wi < nwords) {
                const uint32_t w = (T == 32) ? word32 : (word32 >> (32 - T * (lane + 1))) & ((1u << T) - 1u);
                bits[wi] = (W)w;
            }
        }
    }
}

template <int T>
__global__ void unpack_vec_bits_kernel(const typename TileWord<T>::type* __restrict__ bits,
                                       long long n, float* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t w = bits[i / T];
    out[i] = ((w >> (T - 1 - (int)(i % T))) & 1u) ? 1.0f : 0.0f;
}

b2sr_status launch_pack_vec_bits(const float* x, int n, int T, void* bits, cudaStream_t s) {
    if (n <= 0) return B2SR_SUCCESS;
    const long long nwords = ((long long)n + T - 1) / T;
    const int threads = 256;
    long long blocks = (((long long)n + 31) / 32 * 32 + threads - 1) / threads;
    if (blocks > 65535LL * 8) blocks = 65535LL * 8;
    switch (T) {
        case 4: pack_vec_bits_kernel<4><<<(unsigned)blocks, threads, 0, s>>>(x, n, (uint8_t*)bits, nwords); break;
        case 8: pack_vec_bits_kernel<8><<<(unsigned)blocks, threads, 0, s>>>(x, n, (uint8_t*)bits, nwords); break;
        case 16: pack_vec_bits_kernel<16><<<(unsigned)blocks, threads, 0, s>>>(x, n, (uint16_t*)bits, nwords); break;
        case 32: pack_vec_bits_kernel<32><<<(unsigned)blocks, threads, 0, s>>>(x, n, (uint32_t*)bits, nwords); break;
        default: return B2SR_ERR_INVALID_VALUE;
    }
    B2SR_LAUNCH_CHECK();
    return B2SR_SUCCESS;
}

b2sr_status launch_unpack_vec_bits(const void* bits, int n, int T, float* out, cudaStream_t s) {
    if (n <= 0) return B2SR_SUCCESS;
    const int threads = 256;
    const unsigned blocks = (unsigned)(((long long)n + threads - 1) / threads);
    switch (T) {
        case 4: unpack_vec_bits_kernel<4><<<blocks, threads, 0, s>>>((const uint8_t*)bits, n, out); break;
        case 8: unpack_vec_bits_kernel<8><<<blocks, threads, 0, s>>>((const uint8_t*)bits, n, out); break;
        case 16: unpack_vec_bits_kernel<16><<<blocks, threads, 0, s>>>((const uint16_t*)bits, n, out); break;
        case 32: unpack_vec_bits_kernel<32><<<blocks, threads, 0, s>>>((const uint32_t*)bits, n, out); break;
        default: return B2SR_ERR_INVALID_VALUE;
    }
    B2SR_LAUNCH_CHECK();
    return B2SR_SUCCESS;
}

// ---- set-bit count ----------------------------------------------------------------
__global__ void count_bits_kernel(const uint8_t* __restrict__ bytes, long long nbytes,
                                  unsigned long long* __restrict__ out) {
    unsigned long long c = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nbytes; i += stride)
        c += __popc((unsigned)bytes[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(FULL_MASK, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

b2sr_status launch_count_bits(const void* tiles, long long nwords, int T,
                              unsigned long long* d_count, cudaStream_t s) {
    B2SR_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), s));
    const long long nbytes = nwords * word_bytes(T);
    if (nbytes == 0) return B2SR_SUCCESS;
    const int threads = 256;
    long long blocks = (nbytes + threads - 1) / threads;
    if (blocks > 4096) blocks = 4096;
    count_bits_kernel<<<(unsigned)blocks, threads, 0, s>>>((const uint8_t*)tiles, nbytes, d_count);
    B2SR_LAUNCH_CHECK();
    return B2SR_SUCCESS;
}

}  // namespace b2sr
