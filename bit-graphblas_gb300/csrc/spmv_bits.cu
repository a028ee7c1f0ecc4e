// bin_bin_bin and masked bin_bin_bin instantiations.
#include "b2sr_variants.h"

namespace b2sr {

template <bool MASKED>
static b2sr_status bits_dispatch(int T, const SpmvArgs& args, const LaunchShape& sh, int grid,
                                 cudaStream_t s) {
    switch (T) {
        case 4: return run_merge_shape<OpBits<4, MASKED>, 4>(args, sh, grid, s);
        case 8: return run_merge_shape<OpBits<8, MASKED>, 8>(args, sh, grid, s);
        case 16: return run_merge_shape<OpBits<16, MASKED>, 16>(args, sh, grid, s);
        case 32: return run_merge_shape<OpBits<32, MASKED>, 32>(args, sh, grid, s);
    }
    return B2SR_ERR_INVALID_VALUE;
}

b2sr_status spmv_bits(int T, const SpmvArgs& args, const LaunchShape& sh, int grid, cudaStream_t s) {
    if (args.mask) return bits_dispatch<true>(T, args, sh, grid, s);
    return bits_dispatch<false>(T, args, sh, grid, s);
}

int occupancy_bits(int T, bool masked, const LaunchShape& sh) {
    switch (T) {
        case 4: return masked ? max_ctas_per_sm<OpBits<4, true>, 4>(sh) : max_ctas_per_sm<OpBits<4, false>, 4>(sh);
        case 8: return masked ? max_ctas_per_sm<OpBits<8, true>, 8>(sh) : max_ctas_per_sm<OpBits<8, false>, 8>(sh);
        case 16: return masked ? max_ctas_per_sm<OpBits<16, true>, 16>(sh) : max_ctas_per_sm<OpBits<16, false>, 16>(sh);
        case 32: return masked ? max_ctas_per_sm<OpBits<32, true>, 32>(sh) : max_ctas_per_sm<OpBits<32, false>, 32>(sh);
    }
    return 1;
}

}  // namespace b2sr
