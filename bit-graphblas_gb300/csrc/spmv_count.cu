// bin_bin_full (float counts) and bin_bin_count (int32 counts) instantiations.
#include "b2sr_variants.h"

namespace b2sr {

template <typename Y>
static b2sr_status count_dispatch(int T, const SpmvArgs& args, const LaunchShape& sh, int grid,
                                  cudaStream_t s) {
    switch (T) {
        case 4: return run_merge_shape<OpCount<4, Y>, 4>(args, sh, grid, s);
        case 8: return run_merge_shape<OpCount<8, Y>, 8>(args, sh, grid, s);
        case 16: return run_merge_shape<OpCount<16, Y>, 16>(args, sh, grid, s);
        case 32: return run_merge_shape<OpCount<32, Y>, 32>(args, sh, grid, s);
    }
    return B2SR_ERR_INVALID_VALUE;
}

template <typename Y>
static int count_occupancy(int T, const LaunchShape& sh) {
    switch (T) {
        case 4: return max_ctas_per_sm<OpCount<4, Y>, 4>(sh);
        case 8: return max_ctas_per_sm<OpCount<8, Y>, 8>(sh);
        case 16: return max_ctas_per_sm<OpCount<16, Y>, 16>(sh);
        case 32: return max_ctas_per_sm<OpCount<32, Y>, 32>(sh);
    }
    return 1;
}

b2sr_status spmv_count_f(int T, const SpmvArgs& args, const LaunchShape& sh, int grid, cudaStream_t s) {
    return count_dispatch<float>(T, args, sh, grid, s);
}
b2sr_status spmv_count_i(int T, const SpmvArgs& args, const LaunchShape& sh, int grid, cudaStream_t s) {
    return count_dispatch<int>(T, args, sh, grid, s);
}
int occupancy_count_f(int T, const LaunchShape& sh) { return count_occupancy<float>(T, sh); }
int occupancy_count_i(int T, const LaunchShape& sh) { return count_occupancy<int>(T, sh); }

}  // namespace b2sr
