// bin_bin_bin and masked bin_bin_bin instantiations.
#include "b2sr_spmv_impl.cuh"
#include "b2sr_variants.h"

namespace b2sr {

template <bool MASKED>
static b2sr_status bits_dispatch(const MatView& A, const LaunchShape& sh, int grid,
                                 const Coord* starts, const void* x, void* y, const void* mask,
                                 int accumulate, void* carries, cudaStream_t s) {
    switch (A.T) {
        case 4: return run_merge_shape<OpBits<4, MASKED>, 4>(A, sh, grid, starts, x, y, mask, accumulate, carries, s);
        case 8: return run_merge_shape<OpBits<8, MASKED>, 8>(A, sh, grid, starts, x, y, mask, accumulate, carries, s);
        case 16: return run_merge_shape<OpBits<16, MASKED>, 16>(A, sh, grid, starts, x, y, mask, accumulate, carries, s);
        case 32: return run_merge_shape<OpBits<32, MASKED>, 32>(A, sh, grid, starts, x, y, mask, accumulate, carries, s);
    }
    return B2SR_ERR_INVALID_VALUE;
}

b2sr_status spmv_bits(const MatView& A, const LaunchShape& sh, int grid, const Coord* starts,
                      const void* x, void* y, const void* mask, int accumulate, void* carries,
                      cudaStream_t s) {
    if (mask) return bits_dispatch<true>(A, sh, grid, starts, x, y, mask, 0, carries, s);
    return bits_dispatch<false>(A, sh, grid, starts, x, y, nullptr, accumulate, carries, s);
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
