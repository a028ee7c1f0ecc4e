// Autotuner: picks tile size T, algorithm, gather path and merge-path launch
// shape for one graph and multiply kind by timing candidates on the device.
//
// Decisions are cached in-process per shape key (rows, columns, nonzeros,
// multiply kind, RHS width, SM count) and, when the environment variable
// B2SR_TUNE_CACHE names a file, read from and appended to that file as one
// line per key, so later processes skip the timing.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "b2sr_common.cuh"

namespace b2sr {
namespace {

using TuneKey = std::tuple<int, int, long long, int, int, int>;

std::mutex g_tune_mu;
std::map<TuneKey, b2sr_tune_result> g_tune_cache;
bool g_tune_file_loaded = false;

const char* tune_file() { return std::getenv("B2SR_TUNE_CACHE"); }

void load_tune_file() {
    if (g_tune_file_loaded) return;
    g_tune_file_loaded = true;
    const char* path = tune_file();
    if (!path) return;
    FILE* f = std::fopen(path, "r");
    if (!f) return;
    int nr, nc, var, k, sms;
    long long nnz;
    b2sr_tune_result r;
    std::memset(&r, 0, sizeof r);
    while (std::fscanf(f, "%d %d %lld %d %d %d %d %d %d %d %d %d %f", &nr, &nc, &nnz, &var, &k, &sms, &r.tile_dim,
                       &r.algorithm, &r.gather, &r.threads, &r.items_per_thread, &r.rhs_block, &r.best_ms) == 13) {
        r.candidates = 0;
        g_tune_cache[TuneKey(nr, nc, nnz, var, k, sms)] = r;
    }
    std::fclose(f);
}

void save_tune_line(const TuneKey& key, const b2sr_tune_result& r) {
    const char* path = tune_file();
    if (!path) return;
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%d %d %lld %d %d %d %d %d %d %d %d %d %.6f\n", std::get<0>(key), std::get<1>(key),
                 std::get<2>(key), std::get<3>(key), std::get<4>(key), std::get<5>(key), r.tile_dim, r.algorithm,
                 r.gather, r.threads, r.items_per_thread, r.rhs_block, r.best_ms);
    std::fclose(f);
}

struct Candidate {
    int algorithm, gather, threads, items, rhs_block;
};

std::vector<Candidate> candidates_for(b2sr_variant v, int k) {
    std::vector<Candidate> c;
    if (k > 0) {
        // dense RHS: the narrowest column block covering k, then narrower
        // blocks (more X rows per warp load, more passes over the tiles)
        c.push_back({0, 0, 0, 0, 0});
        for (int blk = 64; blk >= 16; blk /= 2)
            if (blk < k) c.push_back({0, 0, 0, 0, blk});
        return c;
    }
    if (v == B2SR_BIN_FULL_FULL) {
        c.push_back({2, 1, 0, 0, 0});  // row-binned, ld.global gathers
        c.push_back({2, 2, 0, 0, 0});  // row-binned, texture gathers
        c.push_back({2, 3, 0, 0, 0});  // row-binned, set columns only
    } else {
        c.push_back({2, 0, 0, 0, 0});  // row-binned bit-vector kernel
    }
    const int shapes[][2] = {{256, 8}, {256, 4}, {128, 8}, {128, 16}};
    for (auto& sh : shapes) c.push_back({1, 0, sh[0], sh[1], 0});
    return c;
}

// One multiply of the tuned kind on scratch vectors.
b2sr_status run_kind(b2sr_matrix* m, b2sr_variant v, int k, void* x, void* y, cudaStream_t s) {
    if (k > 0) return b2sr_spmm_bin_full_full(m, static_cast<float*>(x), k, k, static_cast<float*>(y), k, 0, s);
    switch (v) {
        case B2SR_BIN_FULL_FULL: return b2sr_spmv_bin_full_full(m, static_cast<float*>(x), static_cast<float*>(y), 0, s);
        case B2SR_BIN_BIN_FULL: return b2sr_spmv_bin_bin_full(m, x, static_cast<float*>(y), 0, s);
        case B2SR_BIN_BIN_COUNT: return b2sr_spmv_bin_bin_count(m, x, static_cast<int*>(y), 0, s);
        case B2SR_BIN_BIN_BIN: return b2sr_spmv_bin_bin_bin(m, x, y, 0, s);
    }
    return B2SR_ERR_INVALID_VALUE;
}

b2sr_status apply(b2sr_matrix* m, b2sr_variant v, const Candidate& c) {
    b2sr_launch_config cfg = {};
    cfg.threads = c.threads;
    cfg.items_per_thread = c.items;
    cfg.ctas_per_sm = 0;
    cfg.algorithm = c.algorithm;
    cfg.gather = c.gather;
    cfg.rhs_block = c.rhs_block;
    cfg.direction = 0;  // pull: the push choice depends on each call's x
    return b2sr_matrix_set_launch(m, v, &cfg);
}

}  // namespace
}  // namespace b2sr

using namespace b2sr;

extern "C" b2sr_status b2sr_autotune(const int* d_rowptr, const int* d_colind, int nrows, int ncols, int nnz,
                                     b2sr_variant variant, int k, const int* tile_dims, int n_tile_dims,
                                     void* stream, b2sr_matrix** out, b2sr_tune_result* result) {
    if (!out || !result || k < 0 || (int)variant < 0 || (int)variant > 3) return B2SR_ERR_INVALID_VALUE;
    if (k > 0 && variant != B2SR_BIN_FULL_FULL) return B2SR_ERR_NOT_SUPPORTED;
    *out = nullptr;
    std::memset(result, 0, sizeof *result);
    static const int default_tiles[] = {4, 8, 16, 32};
    if (!tile_dims || n_tile_dims <= 0) {
        tile_dims = default_tiles;
        n_tile_dims = 4;
    }
    for (int i = 0; i < n_tile_dims; ++i)
        if (!valid_tile(tile_dims[i])) return B2SR_ERR_INVALID_VALUE;
    cudaStream_t s = as_stream(stream);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const TuneKey key(nrows, ncols, (long long)nnz, (int)variant, k, sms);

    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        load_tune_file();
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            b2sr_tune_result r = it->second;
            b2sr_status st = b2sr_pack_csr(d_rowptr, d_colind, nrows, ncols, nnz, r.tile_dim, stream, out);
            if (st != B2SR_SUCCESS) return st;
            st = apply(*out, variant, {r.algorithm, r.gather, r.threads, r.items_per_thread, r.rhs_block});
            if (st != B2SR_SUCCESS) {
                b2sr_free(*out);
                *out = nullptr;
                return st;
            }
            r.candidates = 0;
            *result = r;
            return B2SR_SUCCESS;
        }
    }

    // scratch vectors large enough for every candidate tile size
    const int maxT = 32;
    const long long rows_pad = ((long long)nrows + maxT - 1) / maxT * maxT;
    const long long cols_pad = ((long long)ncols + maxT - 1) / maxT * maxT;
    const int kk = k > 0 ? k : 1;
    const size_t xbytes = (size_t)cols_pad * kk * 4 + 256, ybytes = (size_t)rows_pad * kk * 4 + 256;
    void* x = dev_alloc(xbytes);
    void* y = dev_alloc(ybytes);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!x || !y) {
        dev_free(x);
        dev_free(y);
        return B2SR_ERR_ALLOC;
    }
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemsetAsync(x, 0, xbytes, s);
    cudaMemsetAsync(y, 0, ybytes, s);

    b2sr_status st = B2SR_SUCCESS;
    b2sr_matrix* best = nullptr;
    b2sr_tune_result best_r;
    std::memset(&best_r, 0, sizeof best_r);
    best_r.best_ms = 1e30f;
    int tried = 0;
    const int reps = 7;
    for (int ti = 0; ti < n_tile_dims && st == B2SR_SUCCESS; ++ti) {
        b2sr_matrix* m = nullptr;
        st = b2sr_pack_csr(d_rowptr, d_colind, nrows, ncols, nnz, tile_dims[ti], stream, &m);
        if (st != B2SR_SUCCESS) break;
        bool keep = false;
        for (const Candidate& c : candidates_for(variant, k)) {
            if ((st = apply(m, variant, c)) != B2SR_SUCCESS) break;
            // two untimed runs build the plans and warm the caches
            for (int w = 0; w < 2 && st == B2SR_SUCCESS; ++w) st = run_kind(m, variant, k, x, y, s);
            if (st != B2SR_SUCCESS) break;
            std::vector<float> ms;
            for (int r = 0; r < reps && st == B2SR_SUCCESS; ++r) {
                cudaEventRecord(e0, s);
                st = run_kind(m, variant, k, x, y, s);
                cudaEventRecord(e1, s);
                cudaEventSynchronize(e1);
                float t = 0;
                cudaEventElapsedTime(&t, e0, e1);
                ms.push_back(t);
            }
            if (st != B2SR_SUCCESS) break;
            std::sort(ms.begin(), ms.end());
            const float med = ms[ms.size() / 2];
            ++tried;
            if (med < best_r.best_ms) {
                best_r.best_ms = med;
                best_r.tile_dim = tile_dims[ti];
                best_r.algorithm = c.algorithm;
                best_r.gather = c.gather;
                best_r.threads = c.threads;
                best_r.items_per_thread = c.items;
                best_r.rhs_block = c.rhs_block;
                keep = true;
            }
        }
        if (st != B2SR_SUCCESS) {
            b2sr_free(m);
            break;
        }
        if (keep) {
            if (best) b2sr_free(best);
            best = m;
        } else {
            b2sr_free(m);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamSynchronize(s);
    dev_free(x);
    dev_free(y);
    if (st != B2SR_SUCCESS) {
        if (best) b2sr_free(best);
        return st;
    }
    st = apply(best, variant,
               {best_r.algorithm, best_r.gather, best_r.threads, best_r.items_per_thread, best_r.rhs_block});
    if (st != B2SR_SUCCESS) {
        b2sr_free(best);
        return st;
    }
    best_r.candidates = tried;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = best_r;
        save_tune_line(key, best_r);
    }
    *out = best;
    *result = best_r;
    return B2SR_SUCCESS;
}

extern "C" void b2sr_autotune_clear_cache(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache.clear();
}
