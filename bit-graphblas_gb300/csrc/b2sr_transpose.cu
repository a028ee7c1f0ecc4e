// Transposed B2SR built on the device.
//
// The tiles of A^T, in storage order, are the tiles of A ordered by
// (tile-column, tile-row).  A's tiles are stored in tile-row order, so a
// stable sort of A's tile indices by tile-column gives that order.  The sort
// is a least-significant-digit radix sort over 8-bit digits of the
// tile-column (as many passes as the largest tile-column needs: 3 for the
// 262,144 tile-columns of R-MAT scale 20 at T = 4).  Each pass counts the
// digits of every 2048-tile block, scans the per-(digit, block) counts
// (digit-major, so equal digits keep block order), and scatters: a warp walks
// its 256 consecutive tiles 32 at a time and ranks each tile among the equal
// digits before it with __match_any_sync and a per-warp counter array, so the
// output order is the input order inside every digit (stable).  A^T's rowptr
// is then a lower bound per tile-column in the sorted keys, and one gather
// kernel writes each output tile: a group of T lanes bit-transposes the
// source tile (one ballot per column) and reads the source's tile-row (from
// an array written once, one warp per tile-row), the output tile's column.
//
// Every index a kernel forms stays inside its buffers whatever the column
// values are (digits are masked to 8 bits; the lower bounds are clamped; the
// sorted values are a permutation of the tile indices), and a tile-column
// outside [0, nbc) is reported, not sorted.
#include <algorithm>

#include "b2sr_common.cuh"

namespace b2sr {

namespace {

constexpr int TR_WARPS = 8;                                // warps per block
constexpr int TR_ROUNDS = 8;                               // 32-tile rounds per warp
constexpr int TR_BLOCK = TR_WARPS * 32 * TR_ROUNDS;        // tiles per block
constexpr int TR_RADIX = 256;                              // 8-bit digits

__device__ __forceinline__ int tr_digit(int key, int shift) { return (int)(((unsigned)key >> shift) & (TR_RADIX - 1)); }

// hist[d * nblocks + b] = tiles of block b whose digit is d; the first pass
// also flags tile-columns outside [0, nbc).
__global__ void __launch_bounds__(TR_WARPS * 32)
radix_count_kernel(const int* __restrict__ keys, int n, int shift, int nblocks, int* __restrict__ hist, int nbc,
                   int* __restrict__ bad) {
    __shared__ int cnt[TR_RADIX];
    for (int i = threadIdx.x; i < TR_RADIX; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * TR_BLOCK;
    int flag = 0;
    for (int k = threadIdx.x; k < TR_BLOCK; k += blockDim.x) {
        const long long i = base + k;
        if (i < n) {
            const int key = keys[i];
            if (bad && (unsigned)key >= (unsigned)nbc) flag = 1;
            atomicAdd(&cnt[tr_digit(key, shift)], 1);
        }
    }
    if (flag) atomicOr(bad, 1);
    __syncthreads();
    for (int d = threadIdx.x; d < TR_RADIX; d += blockDim.x) hist[(long long)d * nblocks + blockIdx.x] = cnt[d];
}

// One stable scatter pass.  vals_in == nullptr: the values are the tile
// indices (first pass).  offs = exclusive scan of hist.
__global__ void __launch_bounds__(TR_WARPS * 32)
radix_scatter_kernel(const int* __restrict__ keys_in, const int* __restrict__ vals_in, int n, int shift,
                     int nblocks, const int* __restrict__ offs, int* __restrict__ keys_out,
                     int* __restrict__ vals_out) {
    __shared__ int wcnt[TR_WARPS][TR_RADIX];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < TR_WARPS * TR_RADIX; i += blockDim.x) (&wcnt[0][0])[i] = 0;
    __syncthreads();
    const long long wbase = (long long)blockIdx.x * TR_BLOCK + (long long)warp * 32 * TR_ROUNDS;
    const unsigned below = (1u << lane) - 1u;
    int key[TR_ROUNDS], val[TR_ROUNDS], rank[TR_ROUNDS];
#pragma unroll
    for (int q = 0; q < TR_ROUNDS; ++q) {
        const long long i = wbase + q * 32 + lane;
        const bool ok = i < n;
        key[q] = ok ? keys_in[i] : 0;
        val[q] = ok ? (vals_in ? vals_in[i] : (int)i) : 0;
        // lanes past the end form their own group and count nowhere
        const int d = ok ? tr_digit(key[q], shift) : TR_RADIX;
        const unsigned peers = __match_any_sync(FULL_MASK, d);
        int* c = &wcnt[warp][ok ? d : 0];
        rank[q] = ok ? *c + __popc(peers & below) : 0;
        __syncwarp();
        if (ok && (peers & below) == 0) *c += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per digit: the tiles of the warps before this one come first
    for (int d = threadIdx.x; d < TR_RADIX; d += blockDim.x) {
        int s = 0;
        for (int w = 0; w < TR_WARPS; ++w) {
            const int c = wcnt[w][d];
            wcnt[w][d] = s;
            s += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < TR_ROUNDS; ++q) {
        const long long i = wbase + q * 32 + lane;
        if (i < n) {
            const int d = tr_digit(key[q], shift);
            const int pos = offs[(long long)d * nblocks + blockIdx.x] + wcnt[warp][d] + rank[q];
            keys_out[pos] = key[q];
            vals_out[pos] = val[q];
        }
    }
}

// rowptr_t[c] = first position of tile-column c in the sorted keys (c <= nbc).
__global__ void transpose_rowptr_kernel(const int* __restrict__ keys, int n, int nbc, int* __restrict__ rowptr_t) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c > nbc) return;
    int lo = 0, hi = n;  // first index with keys[idx] >= c
    while (lo < hi) {
        const int mid = lo + ((hi - lo) >> 1);
        if (keys[mid] < c) lo = mid + 1;
        else hi = mid;
    }
    rowptr_t[c] = lo;
}

// tile_row[k] = the tile-row of tile k: one warp per tile-row (grid-stride;
// ranges clamped to [0, nt)).
__global__ void tile_row_kernel(const int* __restrict__ rowptr, int nb, int nt, int* __restrict__ tile_row) {
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nb; r += nwarps) {
        const int b = max(rowptr[r], 0), e = min(rowptr[r + 1], nt);
        for (int k = b + lane; k < e; k += 32) tile_row[k] = (int)r;
    }
}

// Output tile d of A^T from source tile src = order[d] of A (order == nullptr:
// src = d).  One group of T lanes per tile; lane r holds row word r of the
// source.  For output row c the group votes on bit (T-1-c) of every row word;
// the vote of lane r lands at bit r of the group, and reversing T bits puts
// source row r at bit T-1-r (MSB = column 0 of the output tile).  Lane 0 of
// the group writes the output tile's column: the source's tile-row.
__global__ void transpose_gather_kernel(const void* __restrict__ src_tiles, const int* __restrict__ tile_row,
                                        const int* __restrict__ order, int nt, int T, void* __restrict__ dst_tiles,
                                        int* __restrict__ colind_t) {
    const int lane = threadIdx.x & 31;
    const int G = 32 / T;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int g = lane / T, r = lane % T;
    const long long d = warp * G + g;
    const bool valid = d < nt;
    int src = 0;
    uint32_t w = 0;
    if (valid) {
        src = order ? order[d] : (int)d;
        if (T <= 8) w = static_cast<const uint8_t*>(src_tiles)[(long long)src * T + r];
        else if (T == 16) w = static_cast<const uint16_t*>(src_tiles)[(long long)src * T + r];
        else w = static_cast<const uint32_t*>(src_tiles)[(long long)src * T + r];
    }
    uint32_t mine = 0;
    for (int c = 0; c < T; ++c) {
        const unsigned ball = __ballot_sync(FULL_MASK, (w >> (T - 1 - c)) & 1u);
        const uint32_t grp = (T == 32) ? ball : (ball >> (g * T)) & ((1u << T) - 1u);
        const uint32_t rev = __brev(grp) >> (32 - T);
        if (r == c) mine = rev;
    }
    if (!valid) return;
    if (T <= 8) static_cast<uint8_t*>(dst_tiles)[d * T + r] = (uint8_t)mine;
    else if (T == 16) static_cast<uint16_t*>(dst_tiles)[d * T + r] = (uint16_t)mine;
    else static_cast<uint32_t*>(dst_tiles)[d * T + r] = mine;
    if (r == 0) colind_t[d] = tile_row[src];
}

}  // namespace

b2sr_status launch_transpose(const int* rowptr, const int* colind, const void* tiles, int nb, int nbc, int nt, int T,
                             int* rowptr_t, int* colind_t, void* tiles_t, cudaStream_t s) {
    if (nt < 0 || nb < 0 || nbc < 0) return B2SR_ERR_INVALID_VALUE;
    if (nt == 0) {
        B2SR_CUDA_TRY(cudaMemsetAsync(rowptr_t, 0, sizeof(int) * ((size_t)nbc + 1), s));
        return B2SR_SUCCESS;
    }
    if (nb == 0 || nbc == 0) return B2SR_ERR_INVALID_VALUE;  // tiles need a tile-row and a tile-column
    int bits = 0;
    while (bits < 31 && (1LL << bits) < (long long)nbc) ++bits;  // keys < nbc <= 2^bits
    // at least one pass: it also checks every tile-column against nbc
    const int passes = bits > 8 ? (bits + 7) / 8 : 1;
    const int nblocks = (int)(((long long)nt + TR_BLOCK - 1) / TR_BLOCK);
    const int nhist = TR_RADIX * nblocks;
    int* buf[4] = {nullptr, nullptr, nullptr, nullptr};  // keys / values, two of each
    int* hist = nullptr;
    int* flags = nullptr;  // [0] scan overflow, [1] tile-column out of range
    b2sr_status st = B2SR_SUCCESS;
    do {
        for (int*& p : buf) {
            p = static_cast<int*>(dev_alloc(sizeof(int) * (size_t)nt));
            if (!p) { st = B2SR_ERR_ALLOC; break; }
        }
        if (st != B2SR_SUCCESS) break;
        hist = static_cast<int*>(dev_alloc(sizeof(int) * ((size_t)nhist + 1)));
        if (!hist) { st = B2SR_ERR_ALLOC; break; }
        flags = static_cast<int*>(dev_alloc(2 * sizeof(int)));
        if (!flags) { st = B2SR_ERR_ALLOC; break; }
        cudaError_t e = cudaMemsetAsync(flags, 0, 2 * sizeof(int), s);
        if (e != cudaSuccess) { set_cuda_error(e); st = B2SR_ERR_CUDA; break; }
        const int* keys = colind;
        const int* vals = nullptr;
        for (int p = 0; p < passes && st == B2SR_SUCCESS; ++p) {
            const int shift = 8 * p;
            int* ko = buf[(p & 1) * 2];
            int* vo = buf[(p & 1) * 2 + 1];
            radix_count_kernel<<<nblocks, TR_WARPS * 32, 0, s>>>(keys, nt, shift, nblocks, hist, nbc,
                                                                 p == 0 ? flags + 1 : nullptr);
            e = cudaGetLastError();
            if (e != cudaSuccess) { set_cuda_error(e); st = B2SR_ERR_CUDA; break; }
            st = launch_exclusive_scan(hist, nhist, flags, s);  // synchronizes s
            if (st != B2SR_SUCCESS) break;
            radix_scatter_kernel<<<nblocks, TR_WARPS * 32, 0, s>>>(keys, vals, nt, shift, nblocks, hist, ko, vo);
            e = cudaGetLastError();
            if (e != cudaSuccess) { set_cuda_error(e); st = B2SR_ERR_CUDA; break; }
            add_launch_count(4);
            keys = ko;
            vals = vo;
        }
        if (st != B2SR_SUCCESS) break;
        transpose_rowptr_kernel<<<(unsigned)(((long long)nbc + 1 + 255) / 256), 256, 0, s>>>(keys, nt, nbc, rowptr_t);
        // the key buffer the last pass did not write holds the tile-rows
        int* tile_row = buf[(passes & 1) * 2];
        const long long row_blocks = std::min<long long>(((long long)nb * 32 + 255) / 256, 65535LL * 8);
        tile_row_kernel<<<(unsigned)row_blocks, 256, 0, s>>>(rowptr, nb, nt, tile_row);
        const int G = 32 / T;
        const long long warps = ((long long)nt + G - 1) / G;
        transpose_gather_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(tiles, tile_row, vals, nt, T,
                                                                                     tiles_t, colind_t);
        add_launch_count(3);
        e = cudaGetLastError();
        int h[2] = {0, 0};
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, flags, sizeof(h), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { set_cuda_error(e); st = B2SR_ERR_CUDA; break; }
        if (h[1] != 0) st = B2SR_ERR_INVALID_VALUE;  // a tile-column outside the matrix
        else if (h[0] != 0) st = B2SR_ERR_OVERFLOW;
    } while (0);
    // every launch above was followed by a stream synchronization, or failed
    cudaStreamSynchronize(s);
    for (int* p : buf) dev_free(p);
    dev_free(hist);
    dev_free(flags);
    return st;
}

}  // namespace b2sr
