// Per-variant multiply entry points.  Each lives in its own translation unit
// (spmv_*.cu) so the template instantiations compile in parallel.
#pragma once

#include "b2sr_common.cuh"

namespace b2sr {

b2sr_status spmv_full_full(const MatView& A, const LaunchShape& sh, int grid, const Coord* starts,
                           const void* x, void* y, int accumulate, void* carries, cudaStream_t s);
b2sr_status spmv_count_f(const MatView& A, const LaunchShape& sh, int grid, const Coord* starts,
                         const void* x, void* y, int accumulate, void* carries, cudaStream_t s);
b2sr_status spmv_count_i(const MatView& A, const LaunchShape& sh, int grid, const Coord* starts,
                         const void* x, void* y, int accumulate, void* carries, cudaStream_t s);
// mask != nullptr selects the masked BFS-step form (overwrites y).
b2sr_status spmv_bits(const MatView& A, const LaunchShape& sh, int grid, const Coord* starts,
                      const void* x, void* y, const void* mask, int accumulate, void* carries,
                      cudaStream_t s);

int occupancy_full_full(int T, const LaunchShape& sh);
int occupancy_count_f(int T, const LaunchShape& sh);
int occupancy_count_i(int T, const LaunchShape& sh);
int occupancy_bits(int T, bool masked, const LaunchShape& sh);

}  // namespace b2sr
