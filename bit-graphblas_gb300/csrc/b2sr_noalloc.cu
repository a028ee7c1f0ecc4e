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
// it; that first call should therefore come before any stream capture.  The
// cache is keyed by the CUDA context's unique id, so a context created later
// on the same device (after cudaDeviceReset, or a driver-API context) looks
// the address up again instead of using a stale one.  All calls share the one
// array and each call overwrites it, so calls whose GPU work overlaps
// (different streams, no ordering between them) race on it.
#include <cuda.h>

#include <mutex>
#include <vector>

#include "b2sr_common.cuh"

namespace b2sr {
namespace {

// Starts (grid + 1 coordinates) and carries (grid records of 16 + 4T bytes)
// of the merge-path launch; sized for 1200 CTAs at T = 32.
constexpr size_t NOALLOC_SCRATCH_BYTES = 192 * 1024;
__device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

struct NoallocEntry {
    unsigned long long ctx_id;  // unique id of the CUDA context the address belongs to
    int device;
    void* addr;
    int sms;
};
std::mutex g_noalloc_mu;
std::vector<NoallocEntry> g_noalloc;

// Id of the calling thread's current CUDA context (driver entry points taken
// through the runtime, so the library needs no link against libcuda), or 0
// when there is none yet or the driver does not offer the calls.
unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
        cudaGetLastError();
    });
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of g_noalloc_scratch and the SM count of device `dev`
// (which is current), looked up once per CUDA context.
b2sr_status noalloc_setup(int dev, unsigned char** addr, int* sms) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    unsigned long long id = current_context_id();
    if (id != 0) {
        for (const NoallocEntry& e : g_noalloc)
            if (e.ctx_id == id && e.device == dev) {
                *addr = static_cast<unsigned char*>(e.addr);
                *sms = e.sms;
                return B2SR_SUCCESS;
            }
    }
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // also makes the context current
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
    if (id == 0) id = current_context_id();
    // without a context id (driver calls unavailable) nothing is cached: every
    // call looks the address up again
    if (id != 0) g_noalloc.push_back({id, dev, p, n > 0 ? n : 1});
    *addr = static_cast<unsigned char*>(p);
    *sms = n > 0 ? n : 1;
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
    // with rows to compute every array is read: nothing is launched on a null one
    if (!d_x || !d_tiles || !d_colind) return B2SR_ERR_INVALID_VALUE;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return B2SR_ERR_CUDA;
    }
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
