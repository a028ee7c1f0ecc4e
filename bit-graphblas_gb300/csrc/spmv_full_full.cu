// bin_full_full instantiations (FP32 x, FP32 y) for T = 4, 8, 16, 32.
#include "b2sr_variants.h"

namespace b2sr {

b2sr_status spmv_full_full(int T, const SpmvArgs& args, const LaunchShape& sh, int grid, cudaStream_t s) {
    switch (T) {
        case 4: return run_merge_shape<OpFullFull<4>, 4>(args, sh, grid, s);
        case 8: return run_merge_shape<OpFullFull<8>, 8>(args, sh, grid, s);
        case 16: return run_merge_shape<OpFullFull<16>, 16>(args, sh, grid, s);
        case 32: return run_merge_shape<OpFullFull<32>, 32>(args, sh, grid, s);
    }
    return B2SR_ERR_INVALID_VALUE;
}

int occupancy_full_full(int T, const LaunchShape& sh) {
    switch (T) {
        case 4: return max_ctas_per_sm<OpFullFull<4>, 4>(sh);
        case 8: return max_ctas_per_sm<OpFullFull<8>, 8>(sh);
        case 16: return max_ctas_per_sm<OpFullFull<16>, 16>(sh);
        case 32: return max_ctas_per_sm<OpFullFull<32>, 32>(sh);
    }
    return 1;
}

}  // namespace b2sr
