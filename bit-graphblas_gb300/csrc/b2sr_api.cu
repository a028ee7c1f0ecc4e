// C ABI of the B2SR library (include/b2sr.h): matrix handle, packing, vector
// conversion, multiplies and the reference-compatible shims.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "b2sr_common.cuh"

namespace b2sr {

static thread_local int g_last_cuda_error = 0;
static thread_local int g_launches = 0;

void set_cuda_error(cudaError_t e) { g_last_cuda_error = (int)e; }
void set_launch_count(int n) { g_launches = n; }
void add_launch_count(int n) { g_launches += n; }

static std::mutex g_timer_mu;
static std::vector<cudaEvent_t> g_timer_events;  // pairs: [2i] before, [2i+1] after
static int g_timer_capacity = 0, g_timer_next = 0;
static bool g_timer_armed = false, g_timer_open = false;

void kernel_timer_mark(cudaStream_t s, bool begin) {
    std::lock_guard<std::mutex> lk(g_timer_mu);
    if (!g_timer_armed) return;
    if (begin) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
        if (g_timer_next >= g_timer_capacity) return;
        cudaEventRecord(g_timer_events[2 * g_timer_next], s);
        g_timer_open = true;
    } else if (g_timer_open) {
        cudaEventRecord(g_timer_events[2 * g_timer_next + 1], s);
        g_timer_open = false;
        ++g_timer_next;
    }
}

static std::mutex g_alloc_mu;
static b2sr_alloc_fn g_alloc = nullptr;
static b2sr_free_fn g_free = nullptr;
static void* g_alloc_ctx = nullptr;

void* dev_alloc(size_t bytes) {
    if (bytes == 0) bytes = 16;
    b2sr_alloc_fn fn;
    void* ctx;
    {
        std::lock_guard<std::mutex> lk(g_alloc_mu);
        fn = g_alloc;
        ctx = g_alloc_ctx;
    }
    if (fn) return fn(bytes, ctx);
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void dev_free(void* p) {
    if (!p) return;
    b2sr_free_fn fn;
    void* ctx;
    {
        std::lock_guard<std::mutex> lk(g_alloc_mu);
        fn = g_free;
        ctx = g_alloc_ctx;
    }
    if (fn) fn(p, ctx);
    else cudaFree(p);
}

// Per-call scratch: stream-ordered pool memory unless a custom allocator is
// installed (then the allocator's memory, released after the stream drains).
struct Scratch {
    void* ptr = nullptr;
    cudaStream_t stream = nullptr;
    bool pooled = false;
    b2sr_status get(size_t bytes, cudaStream_t s) {
        stream = s;
        bool custom;
        {
            std::lock_guard<std::mutex> lk(g_alloc_mu);
            custom = g_alloc != nullptr;
        }
        if (!custom) {
            cudaError_t e = cudaMallocAsync(&ptr, bytes ? bytes : 16, s);
            if (e != cudaSuccess) {
                set_cuda_error(e);
                cudaGetLastError();
                ptr = nullptr;
                return B2SR_ERR_ALLOC;
            }
            pooled = true;
            return B2SR_SUCCESS;
        }
        ptr = dev_alloc(bytes);
        return ptr ? B2SR_SUCCESS : B2SR_ERR_ALLOC;
    }
    ~Scratch() {
        if (!ptr) return;
        if (pooled) {
            cudaFreeAsync(ptr, stream);
        } else {
            cudaStreamSynchronize(stream);
            dev_free(ptr);
        }
    }
};

static bool stream_capturing(cudaStream_t s) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return cap != cudaStreamCaptureStatusNone;
}

// Scratch of `m` for `stream`, at least `bytes` long.  A buffer that is too
// small is replaced by a larger one; the old one goes to m->retired (a graph
// captured earlier may reference it) and is freed with the matrix.
// While the stream is being captured into a CUDA graph no cudaMalloc is
// allowed: without a large enough cached buffer of this stream, `fallback`
// takes stream-ordered pool memory instead (captured as allocation/free nodes).
static b2sr_status matrix_scratch(const b2sr_matrix* m_const, cudaStream_t s, size_t bytes, void** out,
                                  Scratch& fallback) {
    b2sr_matrix* m = const_cast<b2sr_matrix*>(m_const);
    if (bytes == 0) bytes = 16;
    const bool capturing = stream_capturing(s);
    std::lock_guard<std::mutex> lk(m->scratch_mu);
    for (auto& e : m->scratch) {
        if (e.stream != s) continue;
        if (e.bytes >= bytes) {
            *out = e.ptr;
            return B2SR_SUCCESS;
        }
        if (capturing) break;
        void* p = dev_alloc(bytes);
        if (!p) return B2SR_ERR_ALLOC;
        m->retired.push_back(e.ptr);
        e.ptr = p;
        e.bytes = bytes;
        *out = e.ptr;
        return B2SR_SUCCESS;
    }
    if (capturing) {
        b2sr_status st = fallback.get(bytes, s);
        *out = fallback.ptr;
        return st;
    }
    void* p = dev_alloc(bytes);
    if (!p) return B2SR_ERR_ALLOC;
    m->scratch.push_back({s, p, bytes});
    *out = p;
    return B2SR_SUCCESS;
}

// The row-task SpMM kernel's counters for stream s (see spmm_state): found,
// or allocated and zeroed on s.  During a capture without one, a buffer of
// the graph's own, zeroed inside the graph.
static b2sr_status matrix_spmm_state(const b2sr_matrix* m_const, cudaStream_t s, size_t bytes, void** out,
                                     Scratch& fallback) {
    b2sr_matrix* m = const_cast<b2sr_matrix*>(m_const);
    const bool capturing = stream_capturing(s);
    std::lock_guard<std::mutex> lk(m->scratch_mu);
    for (auto& e : m->spmm_state) {
        if (e.stream != s) continue;
        if (e.bytes >= bytes) {
            *out = e.ptr;
            return B2SR_SUCCESS;
        }
        break;  // the plan's size is fixed, so this does not happen
    }
    void* p = nullptr;
    if (capturing) {
        b2sr_status st = fallback.get(bytes, s);
        if (st != B2SR_SUCCESS) return st;
        p = fallback.ptr;
    } else {
        p = dev_alloc(bytes);
        if (!p) return B2SR_ERR_ALLOC;
    }
    cudaError_t e = cudaMemsetAsync(p, 0, bytes, s);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        if (!capturing) dev_free(p);
        return B2SR_ERR_CUDA;
    }
    if (!capturing) {
        bool replaced = false;
        for (auto& en : m->spmm_state)
            if (en.stream == s) {
                m->retired.push_back(en.ptr);
                en.ptr = p;
                en.bytes = bytes;
                replaced = true;
            }
        if (!replaced) m->spmm_state.push_back({s, p, bytes});
    }
    *out = p;
    return B2SR_SUCCESS;
}

// The auto-direction hints of m (4 ints of mapped host memory, zeroed), or
// null when they cannot be had (the caller then takes the unhinted path).
static int* matrix_auto_hint(b2sr_matrix* m) {
    std::lock_guard<std::mutex> lk(m->scratch_mu);
    if (!m->auto_hint) {
        void* h = nullptr;
        if (cudaHostAlloc(&h, 4 * sizeof(int), cudaHostAllocMapped) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        std::memset(h, 0, 4 * sizeof(int));
        m->auto_hint = static_cast<int*>(h);
    }
    return m->auto_hint;
}

// Side stream, events and zeroed count state of m for stream s (created once).
static b2sr_status matrix_auto_side(b2sr_matrix* m, cudaStream_t s, b2sr_matrix::AutoSide** out) {
    std::lock_guard<std::mutex> lk(m->scratch_mu);
    for (auto& e : m->auto_side)
        if (e.stream == s) {
            *out = &e;
            return B2SR_SUCCESS;
        }
    b2sr_matrix::AutoSide e{s, nullptr, nullptr, nullptr, nullptr};
    cudaError_t err = cudaStreamCreateWithFlags(&e.side, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e.fork, cudaEventDisableTiming);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e.join, cudaEventDisableTiming);
    if (err == cudaSuccess) {
        e.state = static_cast<int*>(dev_alloc(4 * sizeof(int)));
        if (!e.state) err = cudaErrorMemoryAllocation;
    }
    if (err == cudaSuccess) err = cudaMemsetAsync(e.state, 0, 4 * sizeof(int), e.side);
    if (err == cudaSuccess) err = cudaStreamSynchronize(e.side);
    if (err != cudaSuccess) {
        if (e.state) dev_free(e.state);
        if (e.join) cudaEventDestroy(e.join);
        if (e.fork) cudaEventDestroy(e.fork);
        if (e.side) cudaStreamDestroy(e.side);
        set_cuda_error(err);
        return B2SR_ERR_CUDA;
    }
    m->auto_side.push_back(e);
    *out = &m->auto_side.back();
    return B2SR_SUCCESS;
}

static int variant_index(b2sr_variant v) { return (int)v; }

// Default shapes keep the tile-phase parts of one sub-chunk near 32-64 KB of
// shared memory: T*4 bytes per tile for bin_full_full.
static LaunchShape default_shape(b2sr_variant v, int T) {
    LaunchShape s;
    s.threads = 256;
    s.items = 8;
    if (v == B2SR_BIN_FULL_FULL) {
        if (T == 16) s.items = 4;
        if (T == 32) {
            s.threads = 128;
            s.items = 4;
        }
    }
    return s;
}

static bool shape_supported(const LaunchShape& s) {
    return (s.threads == 256 && (s.items == 8 || s.items == 4)) ||
           (s.threads == 128 && (s.items == 16 || s.items == 8 || s.items == 4));
}

static int device_sms(int dev) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

static MatView view_of(const b2sr_matrix* m) {
    MatView v;
    v.rowptr = m->rowptr;
    v.colind = m->colind;
    v.tiles = m->tiles;
    v.nb = m->nb;
    v.ncols = m->ncols;
    v.T = m->T;
    return v;
}

// Grid and CTA start coordinates for (matrix, variant), built on first use.
static std::mutex g_plan_mu;

static b2sr_status get_plan(const b2sr_matrix* m_const, b2sr_variant v, cudaStream_t s,
                            const LaunchPlan** out) {
    b2sr_matrix* m = const_cast<b2sr_matrix*>(m_const);
    std::lock_guard<std::mutex> lk(g_plan_mu);
    LaunchPlan& p = m->plans[variant_index(v)];
    const LaunchShape& want = m->shapes[variant_index(v)];
    if (p.d_starts && p.shape.threads == want.threads && p.shape.items == want.items &&
        p.shape.ctas_per_sm == want.ctas_per_sm) {
        *out = &p;
        return B2SR_SUCCESS;
    }
    // the start coordinates are computed by a kernel on `s`: under capture it
    // would only be recorded, and the cached plan would hold unfilled memory
    if (stream_capturing(s)) return B2SR_ERR_NOT_SUPPORTED;
    if (p.d_starts) {
        m->retired.push_back(p.d_starts);  // a captured graph may still read them
        p.d_starts = nullptr;
    }
    const long long total = (long long)m->nb + m->nt;
    const long long ipc = (long long)want.threads * want.items;
    int grid = merge_grid(v, m->T, want, m->num_sms);
    const long long need = (total + ipc - 1) / ipc;
    if (need < grid) grid = (int)(need > 0 ? need : 1);
    Coord* starts = static_cast<Coord*>(dev_alloc(sizeof(Coord) * ((size_t)grid + 1)));
    if (!starts) return B2SR_ERR_ALLOC;
    b2sr_status st = launch_partition(view_of(m), grid, starts, s);
    if (st != B2SR_SUCCESS) {
        dev_free(starts);
        return st;
    }
    p.shape = want;
    p.grid = grid;
    p.d_starts = starts;
    *out = &p;
    return B2SR_SUCCESS;
}

// Row-binned plans of `m`, built on first use.
// Plans are built from a host copy of rowptr (a synchronizing download), so
// they cannot be built while `s` is being captured: a multiply made during
// capture needs one made on the matrix before it (B2SR_ERR_NOT_SUPPORTED
// otherwise).
static b2sr_status ensure_rowbin(b2sr_matrix* m, cudaStream_t s) {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    if (!m->rowbin_ready) {
        if (stream_capturing(s)) return B2SR_ERR_NOT_SUPPORTED;
        b2sr_status st = rowbin_plan_create(m->rowptr, m->nb, m->T, false, &m->rowbin, s);
        if (st != B2SR_SUCCESS) return st;
        m->rowbin_ready = true;
    }
    return B2SR_SUCCESS;
}

static b2sr_status ensure_rowbin_bits(b2sr_matrix* m, cudaStream_t s) {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    if (!m->rowbin_bits_ready) {
        if (stream_capturing(s)) return B2SR_ERR_NOT_SUPPORTED;
        b2sr_status st = rowbin_plan_create(m->rowptr, m->nb, m->T, true, &m->rowbin_bits, s);
        if (st != B2SR_SUCCESS) return st;
        m->rowbin_bits_ready = true;
    }
    return B2SR_SUCCESS;
}

// The cached transpose for the push direction, built on first use (which
// synchronizes `s`).  *out stays null when it does not exist yet and `s` is
// capturing.
static b2sr_status direction_transpose(b2sr_matrix* m, cudaStream_t s, const b2sr_matrix** out) {
    *out = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_plan_mu);
        if (m->transpose) {
            *out = m->transpose;
            return B2SR_SUCCESS;
        }
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
        cudaGetLastError();
        cap = cudaStreamCaptureStatusNone;
    }
    if (cap != cudaStreamCaptureStatusNone) return B2SR_SUCCESS;
    return b2sr_matrix_transpose(m, s, out);
}

static b2sr_status run_multiply(const b2sr_matrix* m, b2sr_variant v, const void* x, void* y,
                                const void* mask, int accumulate, void* stream) {
    set_launch_count(0);
    if (m && m->nb == 0) return B2SR_SUCCESS;  // no output rows: nothing to write
    if (!m || !y || (!x && m->nt > 0)) return B2SR_ERR_INVALID_VALUE;
    // FP32 x is read in 16-byte segments; y rows are written as float4.
    if (v == B2SR_BIN_FULL_FULL && ((uintptr_t)x % 16 != 0 || (uintptr_t)y % 16 != 0))
        return B2SR_ERR_INVALID_VALUE;
    if ((v == B2SR_BIN_BIN_FULL || v == B2SR_BIN_BIN_COUNT) && (uintptr_t)y % 4 != 0)
        return B2SR_ERR_INVALID_VALUE;
    cudaStream_t s = as_stream(stream);
    if (v != B2SR_BIN_FULL_FULL && m->shapes[variant_index(v)].algorithm != 1) {
        // bit-vector variants on the row-binned plan (default), with the push
        // form over the transpose when the launch shape asks for it
        b2sr_matrix* mm = const_cast<b2sr_matrix*>(m);
        const int kind = v == B2SR_BIN_BIN_BIN ? (mask ? 1 : 0) : v == B2SR_BIN_BIN_COUNT ? 2 : 3;
        int dir = m->shapes[variant_index(v)].direction;
        // FP32 counts are summed by float atomics in the push: exact for
        // integer sums below 2^24 starting from 0, so not with accumulate.
        if (kind == 3 && (accumulate || m->ncols > (1 << 24))) dir = 0;
        if (m->nt == 0) dir = 0;  // nothing to push (and x may be null)
        const b2sr_matrix* t = nullptr;
        if (dir != 0) {
            b2sr_status st = direction_transpose(mm, s, &t);
            if (st != B2SR_SUCCESS) return st;
            if (!t) {
                if (dir == 2) return B2SR_ERR_NOT_SUPPORTED;
                dir = 0;  // auto during capture before the transpose exists
            }
        }
        b2sr_status st = B2SR_SUCCESS;
        if (dir != 2) {
            st = ensure_rowbin_bits(mm, s);
            if (st != B2SR_SUCCESS) return st;
        }
        const size_t pull_bytes = dir == 2 ? 0 : (rowbin_bits_scratch_bytes(m->rowbin_bits, m->T) + 255) / 256 * 256;
        void* scratch = nullptr;
        Scratch fallback;
        st = matrix_scratch(m, s, pull_bytes + (dir ? push_scratch_bytes(m->nbc, m->nt) : 0), &scratch, fallback);
        if (st != B2SR_SUCCESS) return st;
        PushLink link;
        if (dir != 0) {
            // Auto outside a capture: the device's last decision for this kind
            // is a hint.  Hinted pull: the pull alone, with the decision for the
            // next call counted beside it on a side stream.  Otherwise classify
            // and push, and the pull is launched from the device only if the
            // push was not chosen.  Either way the result is the same bits; a
            // wrong hint costs time only.  A capture keeps the host-launched
            // pull that returns when the push ran: a host-side choice would be
            // frozen into the graph, and work after a graph launch does not
            // wait for kernels its nodes launch from the device (measured on
            // GB300), while after an eager launch it does.
            int* hint = (dir == 1 && !stream_capturing(s)) ? matrix_auto_hint(mm) : nullptr;
            int* hint_dev = nullptr;
            if (hint && cudaHostGetDevicePointer(reinterpret_cast<void**>(&hint_dev), hint, 0) != cudaSuccess) {
                cudaGetLastError();
                hint = nullptr;
            }
            if (hint && reinterpret_cast<volatile int*>(hint)[kind] == 2) {
                b2sr_matrix::AutoSide* as = nullptr;
                st = matrix_auto_side(mm, s, &as);
                if (st != B2SR_SUCCESS) return st;
                B2SR_CUDA_TRY(cudaEventRecord(as->fork, s));
                B2SR_CUDA_TRY(cudaStreamWaitEvent(as->side, as->fork, 0));
                st = launch_direction_count(view_of(t), x, m->nt, as->state, hint_dev + kind, as->side);
                if (st != B2SR_SUCCESS) return st;
                B2SR_CUDA_TRY(cudaEventRecord(as->join, as->side));
                st = rowbin_bits(m->rowbin_bits, view_of(m), kind, x, y, mask, accumulate, scratch, PushLink{}, true, s);
                B2SR_CUDA_TRY(cudaStreamWaitEvent(s, as->join, 0));
                return st;
            }
            const size_t y_bytes = kind <= 1 ? (size_t)m->nb * word_bytes(m->T) : (size_t)m->nb * m->T * 4;
            st = launch_push(view_of(t), kind, dir, x, y, mask, accumulate, y_bytes, m->nt,
                             static_cast<char*>(scratch) + pull_bytes, m->num_sms, &link,
                             hint ? hint_dev + kind : nullptr, s);
            if (st != B2SR_SUCCESS || dir == 2) return st;
            link.gate = hint != nullptr;
        }
        st = rowbin_bits(m->rowbin_bits, view_of(m), kind, x, y, mask, accumulate, scratch, link, dir == 0, s);
        if (dir == 1) kernel_timer_mark(s, false);
        return st;
    }
    const LaunchPlan* plan = nullptr;
    b2sr_status st = get_plan(m, v, s, &plan);
    if (st != B2SR_SUCCESS) return st;
    void* carries = nullptr;
    Scratch fallback;
    st = matrix_scratch(m, s, carry_bytes(v, m->T, plan->grid), &carries, fallback);
    if (st != B2SR_SUCCESS) return st;
    return launch_spmv(v, view_of(m), plan->shape, plan->grid, plan->d_starts, x, y, mask,
                       accumulate, carries, s);
}


// bin_full_full through the row-binned kernel.
static b2sr_status run_rowbin(const b2sr_matrix* m_const, const float* x, float* y, int accumulate,
                              void* stream) {
    set_launch_count(0);
    b2sr_matrix* m = const_cast<b2sr_matrix*>(m_const);
    if (m && m->nb == 0) return B2SR_SUCCESS;  // no output rows: nothing to write
    if (!m || !y || (!x && m->nt > 0)) return B2SR_ERR_INVALID_VALUE;
    if ((uintptr_t)x % 16 != 0 || (uintptr_t)y % 16 != 0) return B2SR_ERR_INVALID_VALUE;
    cudaStream_t s = as_stream(stream);
    b2sr_status st = ensure_rowbin(m, s);
    if (st != B2SR_SUCCESS) return st;
    void* partials = nullptr;
    Scratch fallback;
    st = matrix_scratch(m, s, rowbin_scratch_bytes(m->rowbin, m->T, 4), &partials, fallback);
    if (st != B2SR_SUCCESS) return st;
    // T >= 16: only the set columns' x elements by default (R-MAT s20: 0.28 vs
    // 0.34 ms at T = 16, 0.69 vs 1.04 ms at T = 32 on GB300).  T <= 8: whole x
    // segments through the texture path by default (measured faster there);
    // ld.global when asked for or when x cannot back a texture.
    const int gather = m->shapes[B2SR_BIN_FULL_FULL].gather;
    const bool sparse = gather == 3 || (gather == 0 && m->T >= 16);
    const cudaTextureObject_t xtex = (!sparse && gather != 1) ? vector_texture(x, sizeof(float) * (size_t)m->ncols) : 0;
    return rowbin_spmv(m->rowbin, view_of(m), x, y, accumulate, partials, xtex, sparse, s);
}

// Chunk starts of the SpMM work queue, built on first use.
static b2sr_status get_spmm_plan(const b2sr_matrix* m_const, cudaStream_t s, const LaunchPlan** out) {
    b2sr_matrix* m = const_cast<b2sr_matrix*>(m_const);
    std::lock_guard<std::mutex> lk(g_plan_mu);
    LaunchPlan& p = m->spmm_plan;
    if (p.d_starts) {
        *out = &p;
        return B2SR_SUCCESS;
    }
    if (stream_capturing(s)) return B2SR_ERR_NOT_SUPPORTED;  // as get_plan
    const long long total = (long long)m->nb + m->nt;
    const int nchunks = (int)((total + SPMM_CHUNK_ITEMS - 1) / SPMM_CHUNK_ITEMS > 0
                                  ? (total + SPMM_CHUNK_ITEMS - 1) / SPMM_CHUNK_ITEMS : 1);
    Coord* starts = static_cast<Coord*>(dev_alloc(sizeof(Coord) * ((size_t)nchunks + 1)));
    if (!starts) return B2SR_ERR_ALLOC;
    b2sr_status st = launch_partition(view_of(m), nchunks, starts, s);
    if (st != B2SR_SUCCESS) {
        dev_free(starts);
        return st;
    }
    p.grid = nchunks;
    p.d_starts = starts;
    *out = &p;
    return B2SR_SUCCESS;
}

template <typename V>
static b2sr_status run_spmm_api(const b2sr_matrix* m, const V* X, int k, long long ldx, V* Y,
                                long long ldy, int accumulate, void* stream) {
    set_launch_count(0);
    if (m && m->nb == 0 && k >= 0) return B2SR_SUCCESS;  // no output rows
    if (!m || k < 0 || (k > 0 && (!X || !Y)) || ldx < k || ldy < k) return B2SR_ERR_INVALID_VALUE;
    if (k == 0 || m->nb == 0) return B2SR_SUCCESS;
    cudaStream_t s = as_stream(stream);
    void* scratch = nullptr;
    Scratch fallback;
    // row tasks with item lists, unless the bin_full_full launch option asks
    // for the merge path
    if (m->shapes[B2SR_BIN_FULL_FULL].algorithm != 1) {
        b2sr_matrix* mm = const_cast<b2sr_matrix*>(m);
        {
            std::lock_guard<std::mutex> lk(g_plan_mu);
            if (!mm->spmm_rows_ready) {
                if (stream_capturing(s)) return B2SR_ERR_NOT_SUPPORTED;  // as ensure_rowbin
                b2sr_status st = spmm_rows_plan_create(mm->rowptr, mm->tiles, mm->nb, mm->T, mm->num_sms, &mm->spmm_rows, s);
                if (st != B2SR_SUCCESS) return st;
                mm->spmm_rows_ready = true;
            }
        }
        b2sr_status st = matrix_scratch(m, s, spmm_rows_scratch_bytes(m->spmm_rows, m->T, (int)sizeof(V), k),
                                        &scratch, fallback);
        if (st != B2SR_SUCCESS) return st;
        void* state = nullptr;
        Scratch state_fallback;
        st = matrix_spmm_state(m, s, spmm_rows_state_bytes(m->spmm_rows), &state, state_fallback);
        if (st != B2SR_SUCCESS) return st;
        return spmm_rows_launch<V>(view_of(m), m->spmm_rows, X, ldx, Y, ldy, k,
                                   m->shapes[B2SR_BIN_FULL_FULL].rhs_block, accumulate, scratch,
                                   static_cast<int*>(state), m->num_sms, s);
    }
    const LaunchPlan* plan = nullptr;
    b2sr_status st = get_spmm_plan(m, s, &plan);
    if (st != B2SR_SUCCESS) return st;
    st = matrix_scratch(m, s, spmm_scratch_bytes(m->T, (int)sizeof(V), plan->grid, k), &scratch, fallback);
    if (st != B2SR_SUCCESS) return st;
    return spmm_launch<V>(view_of(m), X, ldx, Y, ldy, k, accumulate, plan->d_starts, plan->grid,
                          scratch, spmm_grid_warps(m->num_sms), s);
}

static void free_matrix(b2sr_matrix* m) {
    if (!m) return;
    for (auto& p : m->plans) {
        if (p.d_starts) dev_free(p.d_starts);
        p.d_starts = nullptr;
    }
    if (m->spmm_plan.d_starts) dev_free(m->spmm_plan.d_starts);
    m->spmm_plan.d_starts = nullptr;
    if (m->rowbin_ready) rowbin_plan_free(&m->rowbin);
    m->rowbin_ready = false;
    if (m->rowbin_bits_ready) rowbin_plan_free(&m->rowbin_bits);
    m->rowbin_bits_ready = false;
    if (m->spmm_rows_ready) spmm_rows_plan_free(&m->spmm_rows);
    m->spmm_rows_ready = false;
    for (auto& e : m->scratch) dev_free(e.ptr);
    m->scratch.clear();
    for (auto& e : m->spmm_state) dev_free(e.ptr);
    m->spmm_state.clear();
    for (auto& e : m->auto_side) {
        cudaStreamSynchronize(e.side);
        dev_free(e.state);
        cudaEventDestroy(e.fork);
        cudaEventDestroy(e.join);
        cudaStreamDestroy(e.side);
    }
    m->auto_side.clear();
    if (m->auto_hint) cudaFreeHost(m->auto_hint);
    m->auto_hint = nullptr;
    for (void* p : m->retired) dev_free(p);
    m->retired.clear();
    if (m->owns) {
        dev_free(m->rowptr);
        dev_free(m->colind);
        dev_free(m->tiles);
    }
    if (m->transpose) free_matrix(m->transpose);
    delete m;
}

static b2sr_matrix* new_matrix(int nrows, int ncols, int T) {
    b2sr_matrix* m = new (std::nothrow) b2sr_matrix();
    if (!m) return nullptr;
    m->nrows = nrows;
    m->ncols = ncols;
    m->T = T;
    m->nb = (int)(((long long)nrows + T - 1) / T);
    m->nbc = (int)(((long long)ncols + T - 1) / T);
    int dev = 0;
    cudaGetDevice(&dev);
    m->device = dev;
    m->num_sms = device_sms(dev);
    for (int v = 0; v < 4; ++v) m->shapes[v] = default_shape((b2sr_variant)v, T);
    return m;
}

// Pads an element count so vector loads of the array tail stay inside it.
static size_t padded_bytes(size_t bytes) { return (bytes + 255) / 256 * 256 + 256; }

static b2sr_status count_set_bits(b2sr_matrix* m, cudaStream_t s) {
    unsigned long long* d_cnt = static_cast<unsigned long long*>(dev_alloc(sizeof(unsigned long long)));
    if (!d_cnt) return B2SR_ERR_ALLOC;
    b2sr_status st = launch_count_bits(m->tiles, (long long)m->nt * m->T, m->T, d_cnt, s);
    unsigned long long h = 0;
    if (st == B2SR_SUCCESS) {
        cudaError_t e = cudaMemcpyAsync(&h, d_cnt, sizeof(h), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_cuda_error(e);
            st = B2SR_ERR_CUDA;
        }
    }
    dev_free(d_cnt);
    m->nnz = (long long)h;
    return st;
}

// Validate + count + scan into browptr (nb + 1 entries).  Returns the tile
// count in *nt.  Synchronises `s`.
static b2sr_status structure_pass(const int* rowptr, const int* colind, int nrows, int ncols,
                                  int nnz, int T, int nb, int* browptr, int* nt, cudaStream_t s) {
    int* flags = static_cast<int*>(dev_alloc(2 * sizeof(int)));
    if (!flags) return B2SR_ERR_ALLOC;
    b2sr_status st = B2SR_SUCCESS;
    int h[3] = {0, 0, 0};
    do {
        if (nrows > 0) {
            st = launch_validate_csr(rowptr, colind, nrows, ncols, nnz, flags, s);
            if (st != B2SR_SUCCESS) break;
            st = launch_count_tiles(rowptr, colind, nrows, nb, T, flags, browptr, s);
            if (st != B2SR_SUCCESS) break;
        } else {
            cudaError_t e = cudaMemsetAsync(flags, 0, sizeof(int), s);
            if (e != cudaSuccess) { set_cuda_error(e); st = B2SR_ERR_CUDA; break; }
        }
        st = launch_exclusive_scan(browptr, nb, flags + 1, s);  // synchronises s
        if (st != B2SR_SUCCESS) break;
        cudaError_t e = cudaMemcpy(h, flags, 2 * sizeof(int), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(h + 2, browptr + nb, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { set_cuda_error(e); st = B2SR_ERR_CUDA; break; }
        if (h[0] != 0) { st = B2SR_ERR_INVALID_CSR; break; }
        if (h[1] != 0) { st = B2SR_ERR_OVERFLOW; break; }
        *nt = h[2];
    } while (0);
    dev_free(flags);
    return st;
}

// The shims' fast path.  A kernel-launch shim gets raw B2SR arrays on every
// call, the way the reference drivers launch bmv{T}_* in their timed loops
// (bmv_eval/test_bin_full_full.cu:285-297).  The first call on a set of arrays
// wraps them in a non-owning matrix handle (reading the tile count, which
// synchronizes the device) and builds its row-binned plan; later calls on the
// same arrays reuse both and launch the row-binned kernels with no allocation
// and no host synchronization.  The cache is keyed by (device, rowptr,
// colind, tiles, nblockrows, T): the arrays must not change while an entry
// exists.  b2sr_ref_csr2bsr_nnz / b2sr_ref_csr2bsr_batch drop the entries of
// the arrays they write, and b2sr_ref_release drops entries explicitly.
namespace {
struct ShimEntry {
    int device;
    const void* rowptr;
    const void* colind;
    const void* tiles;
    int nb, T;
    b2sr_matrix* m;
};
std::mutex g_shim_mu;
std::vector<ShimEntry> g_shim;
}  // namespace

// Frees the cached handles whose rowptr, colind or tiles equals one of the
// given pointers (every handle when `all`).  Synchronizes the device first
// when anything is dropped, since kernels in flight may still read its plan.
static void shim_release(const void* a, const void* b, const void* c, bool all) {
    std::vector<b2sr_matrix*> drop;
    {
        std::lock_guard<std::mutex> lk(g_shim_mu);
        auto hit = [&](const ShimEntry& e) {
            if (all) return true;
            for (const void* p : {a, b, c})
                if (p && (p == e.rowptr || p == e.colind || p == e.tiles)) return true;
            return false;
        };
        for (auto it = g_shim.begin(); it != g_shim.end();) {
            if (hit(*it)) {
                drop.push_back(it->m);
                it = g_shim.erase(it);
            } else {
                ++it;
            }
        }
    }
    if (drop.empty()) return;
    cudaDeviceSynchronize();
    for (b2sr_matrix* m : drop) free_matrix(m);
}

}  // namespace b2sr

using namespace b2sr;

extern "C" {

const char* b2sr_status_string(b2sr_status s) {
    switch (s) {
        case B2SR_SUCCESS: return "success";
        case B2SR_ERR_INVALID_VALUE: return "invalid value";
        case B2SR_ERR_INVALID_CSR: return "invalid CSR (rowptr, column range or column order)";
        case B2SR_ERR_ALLOC: return "device allocation failed";
        case B2SR_ERR_CUDA: return "CUDA runtime error";
        case B2SR_ERR_NOT_SUPPORTED: return "not supported";
        case B2SR_ERR_OVERFLOW: return "size exceeds int32 index range";
        case B2SR_ERR_DEVICE_CHECK: return "device-side check failed";
        case B2SR_ERR_IO: return "packed-matrix file missing, short or corrupt";
    }
    return "unknown status";
}

int b2sr_last_cuda_error(void) { return g_last_cuda_error; }
int b2sr_version(void) { return 1 * 10000 + 0 * 100 + 0; }
int b2sr_last_launch_count(void) { return g_launches; }

b2sr_status b2sr_kernel_timer_start(int capacity) {
    if (capacity < 0) return B2SR_ERR_INVALID_VALUE;
    std::lock_guard<std::mutex> lk(g_timer_mu);
    while ((int)g_timer_events.size() < 2 * capacity) {
        cudaEvent_t e = nullptr;
        cudaError_t err = cudaEventCreate(&e);
        if (err != cudaSuccess) {
            set_cuda_error(err);
            return B2SR_ERR_CUDA;
        }
        g_timer_events.push_back(e);
    }
    g_timer_capacity = capacity;
    g_timer_next = 0;
    g_timer_open = false;
    g_timer_armed = capacity > 0;
    return B2SR_SUCCESS;
}

int b2sr_kernel_timer_read(float* ms, int capacity) {
    std::lock_guard<std::mutex> lk(g_timer_mu);
    const int n = std::min(g_timer_next, capacity);
    g_timer_armed = false;
    for (int i = 0; i < n; ++i) {
        cudaError_t e = cudaEventSynchronize(g_timer_events[2 * i + 1]);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[i], g_timer_events[2 * i], g_timer_events[2 * i + 1]);
        if (e != cudaSuccess) {
            set_cuda_error(e);
            return -1;
        }
    }
    g_timer_next = 0;
    return n;
}

void b2sr_set_allocator(b2sr_alloc_fn alloc_fn, b2sr_free_fn free_fn, void* ctx) {
    std::lock_guard<std::mutex> lk(g_alloc_mu);
    if (alloc_fn && free_fn) {
        g_alloc = alloc_fn;
        g_free = free_fn;
        g_alloc_ctx = ctx;
    } else {
        g_alloc = nullptr;
        g_free = nullptr;
        g_alloc_ctx = nullptr;
    }
}

b2sr_status b2sr_pack_csr(const int* d_rowptr, const int* d_colind, int nrows, int ncols, int nnz,
                          int tile_dim, void* stream, b2sr_matrix** out) {
    set_launch_count(0);
    if (!out) return B2SR_ERR_INVALID_VALUE;
    *out = nullptr;
    if (!valid_tile(tile_dim) || nrows < 0 || ncols < 0 || nnz < 0) return B2SR_ERR_INVALID_VALUE;
    if (!d_rowptr || (nnz > 0 && !d_colind)) return B2SR_ERR_INVALID_VALUE;
    cudaStream_t s = as_stream(stream);
    b2sr_matrix* m = new_matrix(nrows, ncols, tile_dim);
    if (!m) return B2SR_ERR_ALLOC;
    m->owns = true;
    b2sr_status st = B2SR_SUCCESS;
    do {
        m->rowptr = static_cast<int*>(dev_alloc(sizeof(int) * ((size_t)m->nb + 1)));
        if (!m->rowptr) { st = B2SR_ERR_ALLOC; break; }
        int nt = 0;
        st = structure_pass(d_rowptr, d_colind, nrows, ncols, nnz, tile_dim, m->nb, m->rowptr, &nt, s);
        if (st != B2SR_SUCCESS) break;
        m->nt = nt;
        const size_t cbytes = padded_bytes(sizeof(int) * (size_t)nt);
        const size_t tbytes = padded_bytes((size_t)nt * tile_dim * word_bytes(tile_dim));
        m->colind = static_cast<int*>(dev_alloc(cbytes));
        m->tiles = dev_alloc(tbytes);
        if (!m->colind || !m->tiles) { st = B2SR_ERR_ALLOC; break; }
        cudaError_t e = cudaMemsetAsync(m->colind, 0, cbytes, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(m->tiles, 0, tbytes, s);
        if (e != cudaSuccess) { set_cuda_error(e); st = B2SR_ERR_CUDA; break; }
        if (nt > 0) {
            st = launch_fill_tiles(d_rowptr, d_colind, nrows, m->nb, tile_dim, m->rowptr, m->colind,
                                   m->tiles, s);
            if (st != B2SR_SUCCESS) break;
        }
        st = count_set_bits(m, s);
    } while (0);
    if (st != B2SR_SUCCESS) {
        cudaStreamSynchronize(s);
        free_matrix(m);
        return st;
    }
    *out = m;
    return B2SR_SUCCESS;
}

b2sr_status b2sr_matrix_wrap(const int* d_rowptr, const int* d_colind, const void* d_tiles,
                             int nrows, int ncols, int nblocks, int tile_dim, void* stream,
                             b2sr_matrix** out) {
    set_launch_count(0);
    if (!out) return B2SR_ERR_INVALID_VALUE;
    *out = nullptr;
    if (!valid_tile(tile_dim) || nrows < 0 || ncols < 0 || nblocks < 0 || !d_rowptr)
        return B2SR_ERR_INVALID_VALUE;
    if (nblocks > 0 && (!d_colind || !d_tiles)) return B2SR_ERR_INVALID_VALUE;
    b2sr_matrix* m = new_matrix(nrows, ncols, tile_dim);
    if (!m) return B2SR_ERR_ALLOC;
    m->owns = false;
    m->rowptr = const_cast<int*>(d_rowptr);
    m->colind = const_cast<int*>(d_colind);
    m->tiles = const_cast<void*>(d_tiles);
    cudaStream_t s = as_stream(stream);
    int last = 0;
    cudaError_t e = cudaMemcpyAsync(&last, d_rowptr + m->nb, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        free_matrix(m);
        return B2SR_ERR_CUDA;
    }
    if (last != nblocks) {
        free_matrix(m);
        return B2SR_ERR_INVALID_VALUE;
    }
    m->nt = nblocks;
    b2sr_status st = count_set_bits(m, s);
    if (st != B2SR_SUCCESS) {
        free_matrix(m);
        return st;
    }
    *out = m;
    return B2SR_SUCCESS;
}

b2sr_status b2sr_matrix_describe(const b2sr_matrix* m, b2sr_matrix_desc* out) {
    if (!m || !out) return B2SR_ERR_INVALID_VALUE;
    out->nrows = m->nrows;
    out->ncols = m->ncols;
    out->tile_dim = m->T;
    out->nblockrows = m->nb;
    out->nblockcols = m->nbc;
    out->nblocks = m->nt;
    out->nnz = m->nnz;
    out->d_rowptr = m->rowptr;
    out->d_colind = m->colind;
    out->d_tiles = m->tiles;
    out->owns_storage = m->owns ? 1 : 0;
    return B2SR_SUCCESS;
}

void b2sr_free(b2sr_matrix* m) {
    if (!m) return;
    cudaDeviceSynchronize();
    free_matrix(m);
}

b2sr_status b2sr_matrix_download(const b2sr_matrix* m, int* h_rowptr, int* h_colind, void* h_tiles) {
    if (!m) return B2SR_ERR_INVALID_VALUE;
    cudaError_t e = cudaSuccess;
    if (h_rowptr) e = cudaMemcpy(h_rowptr, m->rowptr, sizeof(int) * ((size_t)m->nb + 1), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && h_colind && m->nt)
        e = cudaMemcpy(h_colind, m->colind, sizeof(int) * (size_t)m->nt, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && h_tiles && m->nt)
        e = cudaMemcpy(h_tiles, m->tiles, (size_t)m->nt * m->T * word_bytes(m->T), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return B2SR_ERR_CUDA;
    }
    return B2SR_SUCCESS;
}

// ---- packed B2SR files ---------------------------------------------------------------
namespace {
struct PackHeader {
    char magic[8];  // "B2SRPACK"
    uint32_t version;
    int32_t tile_dim, nrows, ncols, nb, nt;
    int64_t nnz;
    uint64_t checksum;  // FNV-1a 64 over rowptr, colind, tiles
    uint32_t reserved[4];  // zero
};
static_assert(sizeof(PackHeader) == 64, "packed header is 64 bytes");

constexpr uint32_t PACK_VERSION = 1;

uint64_t fnv1a(uint64_t h, const void* data, size_t n) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}
constexpr uint64_t FNV_OFFSET = 14695981039346656037ull;
}  // namespace

b2sr_status b2sr_matrix_save(const b2sr_matrix* m, const char* path) {
    if (!m || !path) return B2SR_ERR_INVALID_VALUE;
    const size_t wb = (size_t)word_bytes(m->T);
    std::vector<int> rp((size_t)m->nb + 1), ci((size_t)m->nt);
    std::vector<unsigned char> tl((size_t)m->nt * m->T * wb);
    b2sr_status st = b2sr_matrix_download(m, rp.data(), ci.data(), tl.data());
    if (st != B2SR_SUCCESS) return st;
    PackHeader h;
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, "B2SRPACK", 8);
    h.version = PACK_VERSION;
    h.tile_dim = m->T;
    h.nrows = m->nrows;
    h.ncols = m->ncols;
    h.nb = m->nb;
    h.nt = m->nt;
    h.nnz = m->nnz;
    uint64_t c = fnv1a(FNV_OFFSET, rp.data(), rp.size() * sizeof(int));
    c = fnv1a(c, ci.data(), ci.size() * sizeof(int));
    h.checksum = fnv1a(c, tl.data(), tl.size());
    FILE* f = std::fopen(path, "wb");
    if (!f) return B2SR_ERR_IO;
    bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 &&
              std::fwrite(rp.data(), sizeof(int), rp.size(), f) == rp.size() &&
              (ci.empty() || std::fwrite(ci.data(), sizeof(int), ci.size(), f) == ci.size()) &&
              (tl.empty() || std::fwrite(tl.data(), 1, tl.size(), f) == tl.size());
    ok = (std::fclose(f) == 0) && ok;
    return ok ? B2SR_SUCCESS : B2SR_ERR_IO;
}

b2sr_status b2sr_matrix_load(const char* path, void* stream, b2sr_matrix** out) {
    set_launch_count(0);
    if (!path || !out) return B2SR_ERR_INVALID_VALUE;
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return B2SR_ERR_IO;
    PackHeader h;
    std::vector<int> rp, ci;
    std::vector<unsigned char> tl;
    bool ok = std::fread(&h, sizeof h, 1, f) == 1 && std::memcmp(h.magic, "B2SRPACK", 8) == 0 &&
              h.version == PACK_VERSION && valid_tile(h.tile_dim) && h.nrows >= 0 && h.ncols >= 0 && h.nt >= 0 &&
              h.nb == (int)(((long long)h.nrows + h.tile_dim - 1) / h.tile_dim);
    if (ok) {
        rp.resize((size_t)h.nb + 1);
        ci.resize((size_t)h.nt);
        tl.resize((size_t)h.nt * h.tile_dim * word_bytes(h.tile_dim));
        ok = std::fread(rp.data(), sizeof(int), rp.size(), f) == rp.size() &&
             (ci.empty() || std::fread(ci.data(), sizeof(int), ci.size(), f) == ci.size()) &&
             (tl.empty() || std::fread(tl.data(), 1, tl.size(), f) == tl.size());
    }
    std::fclose(f);
    if (ok) {
        uint64_t c = fnv1a(FNV_OFFSET, rp.data(), rp.size() * sizeof(int));
        c = fnv1a(c, ci.data(), ci.size() * sizeof(int));
        ok = fnv1a(c, tl.data(), tl.size()) == h.checksum;
    }
    // structure: rowptr monotone from 0 to nt, colind in range and ascending per tile-row
    const int nbc = (int)(((long long)h.ncols + h.tile_dim - 1) / h.tile_dim);
    for (int i = 0; ok && i < h.nb; ++i) {
        ok = rp[i] >= 0 && rp[i] <= rp[i + 1] && rp[i + 1] <= h.nt;
        for (int j = rp[i]; ok && j < rp[i + 1]; ++j)
            ok = ci[j] >= 0 && ci[j] < nbc && (j == rp[i] || ci[j - 1] < ci[j]);
    }
    ok = ok && rp[0] == 0 && rp[(size_t)h.nb] == h.nt;
    if (!ok) return B2SR_ERR_IO;
    cudaStream_t s = as_stream(stream);
    b2sr_matrix* m = new_matrix(h.nrows, h.ncols, h.tile_dim);
    if (!m) return B2SR_ERR_ALLOC;
    m->owns = true;
    m->nt = h.nt;
    const size_t cbytes = padded_bytes(sizeof(int) * (size_t)h.nt);
    const size_t tbytes = padded_bytes(tl.size());
    m->rowptr = static_cast<int*>(dev_alloc(sizeof(int) * rp.size()));
    m->colind = static_cast<int*>(dev_alloc(cbytes));
    m->tiles = dev_alloc(tbytes);
    b2sr_status st = B2SR_SUCCESS;
    if (!m->rowptr || !m->colind || !m->tiles) st = B2SR_ERR_ALLOC;
    cudaError_t e = cudaSuccess;
    if (st == B2SR_SUCCESS) {
        e = cudaMemsetAsync(m->colind, 0, cbytes, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(m->tiles, 0, tbytes, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(m->rowptr, rp.data(), sizeof(int) * rp.size(), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && h.nt)
            e = cudaMemcpyAsync(m->colind, ci.data(), sizeof(int) * ci.size(), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && h.nt) e = cudaMemcpyAsync(m->tiles, tl.data(), tl.size(), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // host vectors end here
        if (e != cudaSuccess) {
            set_cuda_error(e);
            st = B2SR_ERR_CUDA;
        }
    }
    if (st == B2SR_SUCCESS) st = count_set_bits(m, s);
    if (st == B2SR_SUCCESS && m->nnz != h.nnz) st = B2SR_ERR_IO;
    if (st != B2SR_SUCCESS) {
        cudaStreamSynchronize(s);
        free_matrix(m);
        return st;
    }
    *out = m;
    return B2SR_SUCCESS;
}

b2sr_status b2sr_matrix_transpose(b2sr_matrix* m, void* stream, const b2sr_matrix** out_t) {
    set_launch_count(0);
    if (!m || !out_t) return B2SR_ERR_INVALID_VALUE;
    {
        std::lock_guard<std::mutex> lk(g_plan_mu);
        if (m->transpose) {
            *out_t = m->transpose;
            return B2SR_SUCCESS;
        }
    }
    cudaStream_t s = as_stream(stream);
    // building it allocates and synchronizes the stream: not inside a capture
    // (nothing is recorded; build it before capturing)
    if (stream_capturing(s)) return B2SR_ERR_NOT_SUPPORTED;
    const int T = m->T, nt = m->nt;
    b2sr_matrix* t = new_matrix(m->ncols, m->nrows, T);
    if (!t) return B2SR_ERR_ALLOC;
    t->owns = true;
    b2sr_status st = B2SR_SUCCESS;
    do {
        t->nt = nt;
        t->rowptr = static_cast<int*>(dev_alloc(sizeof(int) * ((size_t)t->nb + 1)));
        const size_t cbytes = padded_bytes(sizeof(int) * (size_t)nt);
        const size_t tbytes = padded_bytes((size_t)nt * T * word_bytes(T));
        t->colind = static_cast<int*>(dev_alloc(cbytes));
        t->tiles = dev_alloc(tbytes);
        if (!t->rowptr || !t->colind || !t->tiles) { st = B2SR_ERR_ALLOC; break; }
        cudaError_t e = cudaMemsetAsync(t->colind, 0, cbytes, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(t->tiles, 0, tbytes, s);
        if (e != cudaSuccess) { set_cuda_error(e); st = B2SR_ERR_CUDA; break; }
        // tile order of the transpose and the bit transpose of every tile, on
        // the device (synchronizes s)
        st = launch_transpose(m->rowptr, m->colind, m->tiles, m->nb, t->nb, nt, T, t->rowptr, t->colind, t->tiles, s);
        t->nnz = m->nnz;
    } while (0);
    if (st != B2SR_SUCCESS) {
        free_matrix(t);
        return st;
    }
    {
        std::lock_guard<std::mutex> lk(g_plan_mu);
        if (m->transpose) {
            free_matrix(t);
        } else {
            m->transpose = t;
        }
        *out_t = m->transpose;
    }
    return B2SR_SUCCESS;
}

b2sr_status b2sr_pack_vec_bits(const float* d_x, int n, int tile_dim, void* d_bits, void* stream) {
    set_launch_count(0);
    if (!valid_tile(tile_dim) || n < 0) return B2SR_ERR_INVALID_VALUE;
    if (n > 0 && (!d_x || !d_bits)) return B2SR_ERR_INVALID_VALUE;
    b2sr_status st = launch_pack_vec_bits(d_x, n, tile_dim, d_bits, as_stream(stream));
    if (st == B2SR_SUCCESS && n > 0) set_launch_count(1);
    return st;
}

b2sr_status b2sr_unpack_vec_bits(const void* d_bits, int n, int tile_dim, float* d_out, void* stream) {
    set_launch_count(0);
    if (!valid_tile(tile_dim) || n < 0) return B2SR_ERR_INVALID_VALUE;
    if (n > 0 && (!d_bits || !d_out)) return B2SR_ERR_INVALID_VALUE;
    b2sr_status st = launch_unpack_vec_bits(d_bits, n, tile_dim, d_out, as_stream(stream));
    if (st == B2SR_SUCCESS && n > 0) set_launch_count(1);
    return st;
}

b2sr_status b2sr_spmv_bin_bin_bin(const b2sr_matrix* m, const void* d_xbits, void* d_ybits,
                                  int accumulate, void* stream) {
    return run_multiply(m, B2SR_BIN_BIN_BIN, d_xbits, d_ybits, nullptr, accumulate, stream);
}

b2sr_status b2sr_spmv_bin_bin_full(const b2sr_matrix* m, const void* d_xbits, float* d_y,
                                   int accumulate, void* stream) {
    return run_multiply(m, B2SR_BIN_BIN_FULL, d_xbits, d_y, nullptr, accumulate, stream);
}

b2sr_status b2sr_spmv_bin_bin_count(const b2sr_matrix* m, const void* d_xbits, int* d_y,
                                    int accumulate, void* stream) {
    return run_multiply(m, B2SR_BIN_BIN_COUNT, d_xbits, d_y, nullptr, accumulate, stream);
}

b2sr_status b2sr_spmv_bin_full_full(const b2sr_matrix* m, const float* d_x, float* d_y,
                                    int accumulate, void* stream) {
    if (m && m->shapes[B2SR_BIN_FULL_FULL].algorithm != 1)
        return run_rowbin(m, d_x, d_y, accumulate, stream);
    return run_multiply(m, B2SR_BIN_FULL_FULL, d_x, d_y, nullptr, accumulate, stream);
}

b2sr_status b2sr_spmv_multi_bits(const b2sr_matrix* m_const, const void* d_x, void* d_y, int word_bits,
                                  const void* d_mask, int accumulate, void* stream) {
    set_launch_count(0);
    b2sr_matrix* m = const_cast<b2sr_matrix*>(m_const);
    if (word_bits != 32 && word_bits != 64) return B2SR_ERR_INVALID_VALUE;
    if (m && m->nb == 0) return B2SR_SUCCESS;  // no output rows
    if (!m || !d_y || (!d_x && m->nt > 0)) return B2SR_ERR_INVALID_VALUE;
    if ((uintptr_t)d_x % 16 != 0 || (uintptr_t)d_y % 16 != 0 || (uintptr_t)d_mask % 16 != 0)
        return B2SR_ERR_INVALID_VALUE;
    if (d_mask && accumulate) return B2SR_ERR_INVALID_VALUE;
    cudaStream_t s = as_stream(stream);
    b2sr_status st = ensure_rowbin(m, s);
    if (st != B2SR_SUCCESS) return st;
    void* partials = nullptr;
    Scratch fallback;
    st = matrix_scratch(m, s, rowbin_scratch_bytes(m->rowbin, m->T, word_bits / 8), &partials, fallback);
    if (st != B2SR_SUCCESS) return st;
    const cudaTextureObject_t xtex = m->shapes[B2SR_BIN_FULL_FULL].gather != 1
                                         ? vector_texture(d_x, (size_t)word_bits / 8 * (size_t)m->ncols) : 0;
    return rowbin_multi_bits(m->rowbin, view_of(m), d_x, d_y, d_mask, word_bits, accumulate, partials, xtex, s);
}

b2sr_status b2sr_spmv_bin_bin_bin_masked(const b2sr_matrix* m, const void* d_xbits,
                                         const void* d_maskbits, void* d_ybits, void* stream) {
    if (!d_maskbits) return B2SR_ERR_INVALID_VALUE;
    return run_multiply(m, B2SR_BIN_BIN_BIN, d_xbits, d_ybits, d_maskbits, 0, stream);
}

b2sr_status b2sr_spmm_bin_full_full(const b2sr_matrix* m, const float* d_X, int k, long long ldx,
                                    float* d_Y, long long ldy, int accumulate, void* stream) {
    return run_spmm_api<float>(m, d_X, k, ldx, d_Y, ldy, accumulate, stream);
}

b2sr_status b2sr_spmm_bin_full_full_f64(const b2sr_matrix* m, const double* d_X, int k, long long ldx,
                                        double* d_Y, long long ldy, int accumulate, void* stream) {
    return run_spmm_api<double>(m, d_X, k, ldx, d_Y, ldy, accumulate, stream);
}

b2sr_status b2sr_matrix_set_launch(b2sr_matrix* m, b2sr_variant v, const b2sr_launch_config* cfg) {
    if (!m || (int)v < 0 || (int)v > 3) return B2SR_ERR_INVALID_VALUE;
    LaunchShape sh = default_shape(v, m->T);
    if (cfg) {
        if (cfg->threads) sh.threads = cfg->threads;
        if (cfg->items_per_thread) sh.items = cfg->items_per_thread;
        if (cfg->ctas_per_sm < 0 || cfg->algorithm < 0 || cfg->algorithm > 2 || cfg->gather < 0 ||
            cfg->gather > 3 || cfg->direction < 0 || cfg->direction > 2)
            return B2SR_ERR_INVALID_VALUE;
        if (cfg->rhs_block != 0 && cfg->rhs_block != 16 && cfg->rhs_block != 32 && cfg->rhs_block != 64 &&
            cfg->rhs_block != 128)
            return B2SR_ERR_INVALID_VALUE;
        sh.ctas_per_sm = cfg->ctas_per_sm;
        sh.algorithm = cfg->algorithm;
        sh.gather = cfg->gather;
        sh.rhs_block = cfg->rhs_block;
        sh.direction = cfg->direction;
    }
    if (!shape_supported(sh)) return B2SR_ERR_NOT_SUPPORTED;
    std::lock_guard<std::mutex> lk(g_plan_mu);
    m->shapes[variant_index(v)] = sh;
    return B2SR_SUCCESS;
}

b2sr_status b2sr_matrix_get_launch(const b2sr_matrix* m, b2sr_variant v, b2sr_launch_config* cfg) {
    if (!m || !cfg || (int)v < 0 || (int)v > 3) return B2SR_ERR_INVALID_VALUE;
    const LaunchShape& sh = m->shapes[variant_index(v)];
    cfg->threads = sh.threads;
    cfg->items_per_thread = sh.items;
    cfg->ctas_per_sm = sh.ctas_per_sm;
    cfg->algorithm = sh.algorithm;
    cfg->gather = sh.gather;
    cfg->rhs_block = sh.rhs_block;
    cfg->direction = sh.direction;
    return B2SR_SUCCESS;
}

// ---- reference-compatible shims ------------------------------------------------------

b2sr_status b2sr_ref_csr2bsr_nnz(const int* d_csrRowPtr, const int* d_csrColInd, int nrows,
                                 int ncols, int blocksize, int* d_bsrRowPtr, int* h_nblocks) {
    set_launch_count(0);
    if (!valid_tile(blocksize) || nrows < 0 || ncols < 0 || !d_csrRowPtr || !d_bsrRowPtr || !h_nblocks)
        return B2SR_ERR_INVALID_VALUE;
    shim_release(d_bsrRowPtr, nullptr, nullptr, false);  // its rowptr is rewritten
    int nnz = 0;
    cudaError_t e = cudaMemcpy(&nnz, d_csrRowPtr + nrows, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return B2SR_ERR_CUDA;
    }
    const int nb = (int)(((long long)nrows + blocksize - 1) / blocksize);
    return structure_pass(d_csrRowPtr, d_csrColInd, nrows, ncols, nnz, blocksize, nb, d_bsrRowPtr,
                          h_nblocks, nullptr);
}

b2sr_status b2sr_ref_csr2bsr_batch(const int* h_csrRowPtr, const int* h_csrColInd, int nrows,
                                   int ncols, int nnz, int* d_bsrRowPtr, int* d_bsrColInd,
                                   void* d_bsrVal, int blocksize, int nblockrows, int nblocks) {
    set_launch_count(0);
    if (!valid_tile(blocksize) || nrows < 0 || ncols < 0 || nnz < 0 || !h_csrRowPtr || !d_bsrRowPtr)
        return B2SR_ERR_INVALID_VALUE;
    if (nblockrows != (int)(((long long)nrows + blocksize - 1) / blocksize)) return B2SR_ERR_INVALID_VALUE;
    if (nblocks > 0 && (!d_bsrColInd || !d_bsrVal || !h_csrColInd)) return B2SR_ERR_INVALID_VALUE;
    shim_release(d_bsrRowPtr, d_bsrColInd, d_bsrVal, false);  // these arrays are rewritten
    int* d_rp = static_cast<int*>(dev_alloc(sizeof(int) * ((size_t)nrows + 1)));
    int* d_ci = static_cast<int*>(dev_alloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1)));
    b2sr_status st = B2SR_SUCCESS;
    do {
        if (!d_rp || !d_ci) { st = B2SR_ERR_ALLOC; break; }
        cudaError_t e = cudaMemcpy(d_rp, h_csrRowPtr, sizeof(int) * ((size_t)nrows + 1), cudaMemcpyHostToDevice);
        if (e == cudaSuccess && nnz > 0)
            e = cudaMemcpy(d_ci, h_csrColInd, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { set_cuda_error(e); st = B2SR_ERR_CUDA; break; }
        // Re-derive the structure to check it against the caller's rowptr.
        int* chk = static_cast<int*>(dev_alloc(sizeof(int) * ((size_t)nblockrows + 1)));
        if (!chk) { st = B2SR_ERR_ALLOC; break; }
        int nt = 0;
        st = structure_pass(d_rp, d_ci, nrows, ncols, nnz, blocksize, nblockrows, chk, &nt, nullptr);
        dev_free(chk);
        if (st != B2SR_SUCCESS) break;
        if (nt != nblocks) { st = B2SR_ERR_INVALID_VALUE; break; }
        if (nblocks > 0) {
            e = cudaMemset(d_bsrVal, 0, (size_t)nblocks * blocksize * word_bytes(blocksize));
            if (e != cudaSuccess) { set_cuda_error(e); st = B2SR_ERR_CUDA; break; }
            st = launch_fill_tiles(d_rp, d_ci, nrows, nblockrows, blocksize, d_bsrRowPtr, d_bsrColInd,
                                   d_bsrVal, nullptr);
            if (st != B2SR_SUCCESS) break;
            e = cudaDeviceSynchronize();
            if (e != cudaSuccess) { set_cuda_error(e); st = B2SR_ERR_CUDA; break; }
        }
    } while (0);
    dev_free(d_rp);
    dev_free(d_ci);
    return st;
}

static b2sr_status ref_multiply(b2sr_variant v, int T, const void* A, const void* B, void* C,
                                const int* rowptr, const int* colind, int nblockrows) {
    set_launch_count(0);
    if (!valid_tile(T) || nblockrows < 0 || !rowptr || !C) return B2SR_ERR_INVALID_VALUE;
    if (nblockrows == 0) return B2SR_SUCCESS;
    // with rows to compute every array is read: nothing is launched on a null one
    if (!A || !B || !colind) return B2SR_ERR_INVALID_VALUE;
    // FP32 x is read in 16-byte segments and y rows written as float4
    if (v == B2SR_BIN_FULL_FULL && ((uintptr_t)B % 16 != 0 || (uintptr_t)C % 16 != 0)) return B2SR_ERR_INVALID_VALUE;
    if (v == B2SR_BIN_BIN_FULL && (uintptr_t)C % 4 != 0) return B2SR_ERR_INVALID_VALUE;
    if ((long long)nblockrows * T > INT_MAX) return B2SR_ERR_OVERFLOW;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return B2SR_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_shim_mu);
    b2sr_matrix* m = nullptr;
    for (const ShimEntry& se : g_shim)
        if (se.device == dev && se.rowptr == rowptr && se.colind == colind && se.tiles == A &&
            se.nb == nblockrows && se.T == T) {
            m = se.m;
            break;
        }
    if (!m) {
        // the reference's matrices are square with x padded to nb*T entries
        m = new_matrix(nblockrows * T, nblockrows * T, T);
        if (!m) return B2SR_ERR_ALLOC;
        m->owns = false;
        m->rowptr = const_cast<int*>(rowptr);
        m->colind = const_cast<int*>(colind);
        m->tiles = const_cast<void*>(A);
        int nt = 0;
        e = cudaMemcpy(&nt, rowptr + nblockrows, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess || nt < 0) {
            if (e != cudaSuccess) set_cuda_error(e);
            free_matrix(m);
            return e != cudaSuccess ? B2SR_ERR_CUDA : B2SR_ERR_INVALID_VALUE;
        }
        m->nt = nt;
        g_shim.push_back({dev, rowptr, colind, A, nblockrows, T, m});
    }
    // the reference kernels accumulate (+= and |=) on the legacy default stream
    if (v == B2SR_BIN_FULL_FULL) return run_rowbin(m, static_cast<const float*>(B), static_cast<float*>(C), 1, nullptr);
    return run_multiply(m, v, B, C, nullptr, 1, nullptr);
}

b2sr_status b2sr_ref_bmv_bin_bin_bin(int tile_dim, const void* A, const void* B, void* C,
                                     const int* rowptr, const int* colind, int nblockrows) {
    return ref_multiply(B2SR_BIN_BIN_BIN, tile_dim, A, B, C, rowptr, colind, nblockrows);
}

b2sr_status b2sr_ref_bmv_bin_bin_full(int tile_dim, const void* A, const void* B, float* C,
                                      const int* rowptr, const int* colind, int nblockrows) {
    return ref_multiply(B2SR_BIN_BIN_FULL, tile_dim, A, B, C, rowptr, colind, nblockrows);
}

b2sr_status b2sr_ref_bmv_bin_full_full(int tile_dim, const void* A, const float* B, float* C,
                                       const int* rowptr, const int* colind, int nblockrows) {
    return ref_multiply(B2SR_BIN_FULL_FULL, tile_dim, A, B, C, rowptr, colind, nblockrows);
}

void b2sr_ref_release(const int* rowptr) { shim_release(rowptr, nullptr, nullptr, rowptr == nullptr); }

}  // extern "C"
