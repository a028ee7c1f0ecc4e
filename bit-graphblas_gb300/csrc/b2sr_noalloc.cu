// Allocation-free bin_full_full multiply on raw B2SR arrays.
//
// Some callers cannot allocate device memory at the moment they multiply:
// processes whose device-memory budget is fully reserved up front, real-time
// loops where a cudaMalloc/cudaFree would stall (cudaFree synchronizes the
// device), and hosts that route every allocation through their own pool and
// forbid the CUDA allocator.  For them this entry point takes its scratch (the
// merge-path start coordinate of every CTA and the CTAs' carries) from a
// fixed array in device memory that the library declares at file scope: every
// GPU that loads the library holds NOALLOC_SCRATCH_BYTES of it until exit.
//
// Host code cannot use the array's name as a device address (in host code it
// names a host-side stand-in).  The first call on each device, with that
// device current, looks the address up with cudaGetSymbolAddress and caches
// it; that first call should therefore come before any stream capture.  All
// calls share the one array and each call overwrites it, so calls whose GPU
// work overlaps (different streams, no ordering between them) race on it.
#include <mutex>

#include "b2sr_common.cuh"

namespace b2sr {
namespace {

// Starts (grid + 1 coordinates) and carries (grid records of 16 + 4T bytes)
// of the merge-path launch; sized for 1200 CTAs at T = 32.
constexpr size_t NOALLOC_SCRATCH_BYTES = 192 * 1024;
__device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};
int g_noalloc_sms[NOALLOC_MAX_DEVICES] = {};

// Device address of g_noalloc_scratch and the SM count of device `dev`
// (which is current), looked up once per device.
b2sr_status noalloc_setup(int dev, unsigned char** addr, int* sms) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            set_cuda_error(e);
            cudaGetLastError();
            return B2SR_ERR_CUDA;
        }
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) {
            set_cuda_error(e);
            cudaGetLastError();
            return B2SR_ERR_CUDA;
        }
        g_noalloc_sms[dev] = n > 0 ? n : 1;
        g_noalloc_addr[dev] = p;
    }
    *addr = static_cast<unsigned char*>(g_noalloc_addr[dev]);
    *sms = g_noalloc_sms[dev];
    return B2SR_SUCCESS;
}

}  // namespace
}  // namespace b2sr

using namespace b2sr;

extern "C" b2sr_status b2sr_spmv_bin_full_full_noalloc(int tile_dim, const void* d_tiles, const int* d_rowptr,
                                                       const int* d_colind, int nblockrows, int ncols,
                                                       const float* d_x, float* d_y, int accumulate,
                                                       void* stream) {
    set_launch_count(0);
    if (!valid_tile(tile_dim) || nblockrows < 0 || ncols < 0 || !d_rowptr || !d_y) return B2SR_ERR_INVALID_VALUE;
    if ((uintptr_t)d_x % 16 != 0 || (uintptr_t)d_y % 16 != 0) return B2SR_ERR_INVALID_VALUE;
    if (nblockrows == 0) return B2SR_SUCCESS;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return B2SR_ERR_CUDA;
    }
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return B2SR_ERR_NOT_SUPPORTED;
    unsigned char* scratch = nullptr;
    int sms = 0;
    b2sr_status st = noalloc_setup(dev, &scratch, &sms);
    if (st != B2SR_SUCCESS) return st;

    // the merge-path shape the matrix API uses for bin_full_full by default
    LaunchShape shape;
    shape.threads = tile_dim == 32 ? 128 : 256;
    shape.items = tile_dim >= 16 ? 4 : 8;
    const int grid = merge_grid(B2SR_BIN_FULL_FULL, tile_dim, shape, sms);
    const size_t starts_bytes = ((size_t)(grid + 1) * sizeof(Coord) + 255) / 256 * 256;
    const size_t need = starts_bytes + carry_bytes(B2SR_BIN_FULL_FULL, tile_dim, grid);
    if (need > NOALLOC_SCRATCH_BYTES) return B2SR_ERR_NOT_SUPPORTED;  // device too large for the fixed scratch

    MatView view;
    view.rowptr = d_rowptr;
    view.colind = d_colind;
    view.tiles = d_tiles;
    view.nb = nblockrows;
    view.ncols = ncols;
    view.T = tile_dim;
    cudaStream_t s = as_stream(stream);
    Coord* starts = reinterpret_cast<Coord*>(scratch);
    st = launch_partition(view, grid, starts, s);
    if (st != B2SR_SUCCESS) return st;
    // every CTA writes its own carry record, so nothing needs clearing first
    return launch_spmv(B2SR_BIN_FULL_FULL, view, shape, grid, starts, d_x, d_y, nullptr, accumulate,
                       scratch + starts_bytes, s);
}
