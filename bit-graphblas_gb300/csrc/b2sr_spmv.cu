// Multiply dispatch: partition kernel, variant/tile-size dispatch, scratch sizing.
#include "b2sr_variants.h"

namespace b2sr {

__global__ void partition_kernel(const int* __restrict__ rowptr, int nb, int grid,
                                 Coord* __restrict__ starts) {
    const int lane = threadIdx.x & 31;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c > grid) return;
    const long long nt = rowptr[nb];
    const long long total = (long long)nb + nt;
    const long long d = total * c / grid;
    long long lo = d - nt > 0 ? d - nt : 0;
    long long hi = d < nb ? d : nb;
    // Invariant: the answer lies in [lo, hi].
    while (hi - lo > 32) {
        const long long span = hi - lo;
        const long long p = lo + (span * (lane + 1)) / 33;
        const bool pred = rowptr[p + 1] <= d - p - 1;
        const unsigned ball = __ballot_sync(FULL_MASK, pred);
        const int t = __popc(ball);  // predicate is monotone: the first t probes are true
        const long long p_last_true = lo + (span * t) / 33;          // probe t-1 (lane t-1)
        const long long p_first_false = lo + (span * (t + 1)) / 33;  // probe t (lane t)
        if (t > 0) lo = p_last_true + 1;
        if (t < 32) hi = p_first_false;
    }
    const long long p = lo + lane;
    const bool pred = p < hi && rowptr[p + 1] <= d - p - 1;
    const int t = __popc(__ballot_sync(FULL_MASK, pred));
    if (lane == 0) {
        const long long x = lo + t;
        starts[c].row = (int)x;
        starts[c].tile = (int)(d - x);
    }
}

b2sr_status launch_partition(const MatView& A, int grid, Coord* d_starts, cudaStream_t s) {
    const int threads = 128;
    const long long warps = (long long)grid + 1;
    const unsigned blocks = (unsigned)((warps * 32 + threads - 1) / threads);
    partition_kernel<<<blocks, threads, 0, s>>>(A.rowptr, A.nb, grid, d_starts);
    B2SR_LAUNCH_CHECK();
    add_launch_count(1);
    return B2SR_SUCCESS;
}

static int ctas_per_sm(b2sr_variant v, int T, const LaunchShape& shape) {
    switch (v) {
        case B2SR_BIN_FULL_FULL: return occupancy_full_full(T, shape);
        case B2SR_BIN_BIN_FULL: return occupancy_count_f(T, shape);
        case B2SR_BIN_BIN_COUNT: return occupancy_count_i(T, shape);
        case B2SR_BIN_BIN_BIN: return occupancy_bits(T, false, shape);
    }
    return 1;
}

int merge_grid(b2sr_variant v, int T, const LaunchShape& shape, int num_sms) {
    int per_sm = ctas_per_sm(v, T, shape);
    if (shape.ctas_per_sm > 0 && shape.ctas_per_sm < per_sm) per_sm = shape.ctas_per_sm;
    return num_sms * per_sm;
}

size_t carry_bytes(b2sr_variant v, int T, int grid) {
    size_t rec = 0;
    switch (v) {
        case B2SR_BIN_FULL_FULL: rec = 16 + 4 * (size_t)T; break;
        case B2SR_BIN_BIN_FULL:
        case B2SR_BIN_BIN_COUNT: rec = 16 + 4 * (size_t)T; break;
        case B2SR_BIN_BIN_BIN: rec = 32; break;
    }
    rec = (rec + 15) / 16 * 16;
    return rec * (size_t)(grid > 0 ? grid : 1);
}

b2sr_status launch_spmv(b2sr_variant v, const MatView& A, const LaunchShape& shape, int grid,
                        const Coord* d_starts, const void* x, void* y, const void* mask,
                        int accumulate, void* carries, cudaStream_t s) {
    SpmvArgs args;
    args.rowptr = A.rowptr;
    args.colind = A.colind;
    args.tiles = A.tiles;
    args.x = x;
    args.y = y;
    args.mask = mask;
    args.starts = d_starts;
    args.carries = carries;
    args.nb = A.nb;
    args.ncols = A.ncols;
    args.accumulate = accumulate;
    switch (v) {
        case B2SR_BIN_FULL_FULL: return spmv_full_full(A.T, args, shape, grid, s);
        case B2SR_BIN_BIN_FULL: return spmv_count_f(A.T, args, shape, grid, s);
        case B2SR_BIN_BIN_COUNT: return spmv_count_i(A.T, args, shape, grid, s);
        case B2SR_BIN_BIN_BIN: return spmv_bits(A.T, args, shape, grid, s);
    }
    return B2SR_ERR_INVALID_VALUE;
}

}  // namespace b2sr
