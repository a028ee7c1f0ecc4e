// Per-variant multiply entry points.  Each lives in its own translation unit
// (spmv_*.cu) so the template instantiations compile in parallel.
#pragma once

#include "b2sr_spmv_impl.cuh"

namespace b2sr {

b2sr_status spmv_full_full(int T, const SpmvArgs& args, const LaunchShape& sh, int grid, cudaStream_t s);
b2sr_status spmv_count_f(int T, const SpmvArgs& args, const LaunchShape& sh, int grid, cudaStream_t s);
b2sr_status spmv_count_i(int T, const SpmvArgs& args, const LaunchShape& sh, int grid, cudaStream_t s);
// args.mask != nullptr selects the masked BFS-step form (overwrites y).
b2sr_status spmv_bits(int T, const SpmvArgs& args, const LaunchShape& sh, int grid, cudaStream_t s);

int occupancy_full_full(int T, const LaunchShape& sh);
int occupancy_count_f(int T, const LaunchShape& sh);
int occupancy_count_i(int T, const LaunchShape& sh);
int occupancy_bits(int T, bool masked, const LaunchShape& sh);

}  // namespace b2sr
