// Host-side graph ingest (include/b2sr_graph.h): canonical CSR construction,
// seeded R-MAT / Erdos-Renyi generators, block-diagonal stacking and a Matrix
// Market reader.  Parallel with OpenMP; results do not depend on the thread
// count.
#include "../../include/b2sr_graph.h"

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// splitmix64 finaliser (Steele, Lea & Flood, "Fast splittable pseudorandom
// number generators", OOPSLA 2014).
inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Counter-based uniform double in [0, 1): draw k of stream `seed`.
inline double uniform_at(uint64_t seed_key, uint64_t k) {
    const uint64_t z = mix64(seed_key + k * 0xD1B54A32D192ED03ull);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

inline uint64_t seed_key(uint64_t seed) { return mix64(seed ^ 0x5851F42D4C957F2Dull); }

bool alloc_csr(int nrows, int ncols, long long nnz, b2sr_csr_host* out) {
    out->nrows = nrows;
    out->ncols = ncols;
    out->nnz = nnz;
    out->rowptr = static_cast<int*>(std::malloc(sizeof(int) * ((size_t)nrows + 1)));
    out->colind = static_cast<int*>(std::malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1)));
    if (!out->rowptr || !out->colind) {
        std::free(out->rowptr);
        std::free(out->colind);
        out->rowptr = out->colind = nullptr;
        return false;
    }
    return true;
}

// Canonical CSR from an edge list given as a callback (u, v) over [0, nedges).
template <class EdgeFn>
int build_canonical(EdgeFn edge, long long nedges, int nrows, int ncols, bool symmetrize,
                    bool drop_self, b2sr_csr_host* out) {
    std::vector<long long> cnt((size_t)nrows + 1, 0);
    // Pass 1: entries per row.
#pragma omp parallel for schedule(static)
    for (long long e = 0; e < nedges; ++e) {
        int u, v;
        edge(e, u, v);
        if (u == v && drop_self) continue;
        __atomic_fetch_add(&cnt[(size_t)u], 1LL, __ATOMIC_RELAXED);
        if (symmetrize && u != v) __atomic_fetch_add(&cnt[(size_t)v], 1LL, __ATOMIC_RELAXED);
    }
    std::vector<long long> off((size_t)nrows + 1, 0);
    for (int i = 0; i < nrows; ++i) off[(size_t)i + 1] = off[i] + cnt[i];
    const long long total = off[nrows];
    std::vector<int> buf((size_t)(total > 0 ? total : 1));
    std::vector<long long> pos(off.begin(), off.end() - 1);
    // Pass 2: scatter (order inside a row is fixed by the sort below).
#pragma omp parallel for schedule(static)
    for (long long e = 0; e < nedges; ++e) {
        int u, v;
        edge(e, u, v);
        if (u == v && drop_self) continue;
        buf[(size_t)__atomic_fetch_add(&pos[(size_t)u], 1LL, __ATOMIC_RELAXED)] = v;
        if (symmetrize && u != v)
            buf[(size_t)__atomic_fetch_add(&pos[(size_t)v], 1LL, __ATOMIC_RELAXED)] = u;
    }
    // Pass 3: sort and de-duplicate every row.
    std::vector<long long> kept((size_t)nrows + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int i = 0; i < nrows; ++i) {
        int* b = buf.data() + off[i];
        int* e = buf.data() + off[(size_t)i + 1];
        std::sort(b, e);
        kept[(size_t)i + 1] = std::unique(b, e) - b;
    }
    for (int i = 0; i < nrows; ++i) kept[(size_t)i + 1] += kept[i];
    const long long nnz = kept[nrows];
    if (nnz > INT_MAX) return 4;
    if (!alloc_csr(nrows, ncols, nnz, out)) return 5;
    for (int i = 0; i <= nrows; ++i) out->rowptr[i] = (int)kept[i];
#pragma omp parallel for schedule(dynamic, 1024)
    for (int i = 0; i < nrows; ++i) {
        const long long n = kept[(size_t)i + 1] - kept[i];
        if (n) std::memcpy(out->colind + kept[i], buf.data() + off[i], sizeof(int) * (size_t)n);
    }
    return 0;
}

}  // namespace

extern "C" {

void b2sr_graph_free(b2sr_csr_host* g) {
    if (!g) return;
    std::free(g->rowptr);
    std::free(g->colind);
    g->rowptr = g->colind = nullptr;
    g->nnz = 0;
}

void b2sr_graph_uniform(uint64_t seed, long long first, long long count, double* out) {
    const uint64_t key = seed_key(seed);
    for (long long i = 0; i < count; ++i) out[i] = uniform_at(key, (uint64_t)(first + i));
}

int b2sr_graph_coo_to_csr(const int* rows, const int* cols, long long nedges, int nrows, int ncols,
                          int symmetrize, int drop_self_loops, b2sr_csr_host* out) {
    if (!out || nrows < 0 || ncols < 0 || nedges < 0 || (nedges > 0 && (!rows || !cols))) return 1;
    for (long long e = 0; e < nedges; ++e)
        if (rows[e] < 0 || rows[e] >= nrows || cols[e] < 0 || cols[e] >= ncols ||
            (symmetrize && (cols[e] >= nrows || rows[e] >= ncols)))
            return 3;
    auto edge = [&](long long e, int& u, int& v) {
        u = rows[e];
        v = cols[e];
    };
    return build_canonical(edge, nedges, nrows, ncols, symmetrize != 0, drop_self_loops != 0, out);
}

int b2sr_graph_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed,
                    b2sr_csr_host* out) {
    if (!out || scale < 1 || scale > 30 || edge_factor < 1) return 1;
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return 1;
    const int n = 1 << scale;
    const long long m = (long long)edge_factor << scale;
    const uint64_t key = seed_key(seed);
    const double ab = a + b, abc = a + b + c;
    // Edge e descends `scale` levels of the adjacency quadtree; level l picks a
    // quadrant with draw e*scale + l and sets bit (scale-1-l) of both ends.
    auto edge = [&](long long e, int& u, int& v) {
        int uu = 0, vv = 0;
        for (int l = 0; l < scale; ++l) {
            const double r = uniform_at(key, (uint64_t)e * (uint64_t)scale + (uint64_t)l);
            const int bit = scale - 1 - l;
            if (r < a) {
            } else if (r < ab) {
                vv |= 1 << bit;
            } else if (r < abc) {
                uu |= 1 << bit;
            } else {
                uu |= 1 << bit;
                vv |= 1 << bit;
            }
        }
        u = uu;
        v = vv;
    };
    return build_canonical(edge, m, n, n, true, true, out);
}

int b2sr_graph_er(int n, long long m, uint64_t seed, b2sr_csr_host* out) {
    if (!out || n < 0 || m < 0) return 1;
    if (n < 2 && m > 0) return 1;
    if ((double)m > 0.5 * (double)n * (double)(n - 1)) return 1;
    const uint64_t key = seed_key(seed);
    // Candidate k is the pair (floor(U_2k n), floor(U_2k+1 n)); the first m
    // distinct unordered pairs of the stream are kept.
    std::unordered_set<uint64_t> seen;
    seen.reserve((size_t)m * 2 + 16);
    std::vector<int> us, vs;
    us.reserve((size_t)m);
    vs.reserve((size_t)m);
    for (uint64_t k = 0; (long long)us.size() < m; ++k) {
        int u = (int)(uniform_at(key, 2 * k) * n);
        int v = (int)(uniform_at(key, 2 * k + 1) * n);
        if (u >= n) u = n - 1;
        if (v >= n) v = n - 1;
        if (u == v) continue;
        if (u > v) std::swap(u, v);
        const uint64_t pk = ((uint64_t)u << 32) | (uint64_t)v;
        if (seen.insert(pk).second) {
            us.push_back(u);
            vs.push_back(v);
        }
    }
    auto edge = [&](long long e, int& u, int& v) {
        u = us[(size_t)e];
        v = vs[(size_t)e];
    };
    return build_canonical(edge, m, n, n, true, true, out);
}

int b2sr_graph_er_batch(int count, double n_min, double n_max, double deg_min, double deg_max, int align,
                        uint64_t seed, b2sr_csr_host* out, int* offsets, int* sizes, double* degrees) {
    if (!out || !offsets || count < 0 || n_min < 2 || n_max < n_min || deg_min < 0 || deg_max < deg_min ||
        align < 1)
        return 1;
    // graph g: n_g = round(exp(U[ln n_min, ln n_max])), degree d_g = U[deg_min, deg_max],
    // m_g = round(n_g * d_g / 2) pairs, seed = seed * 1000 + g; draws from a
    // stream keyed by `seed` (2g: size, 2g+1: degree)
    const uint64_t key = seed_key(seed);
    std::vector<int> n(count);
    std::vector<long long> m(count);
    for (int g = 0; g < count; ++g) {
        const double u = uniform_at(key, 2 * (uint64_t)g), v = uniform_at(key, 2 * (uint64_t)g + 1);
        n[g] = (int)std::llround(std::exp(std::log(n_min) + u * (std::log(n_max) - std::log(n_min))));
        const double d = deg_min + v * (deg_max - deg_min);
        m[g] = std::min((long long)std::llround(n[g] * d / 2.0), (long long)n[g] * (n[g] - 1) / 2);
        if (sizes) sizes[g] = n[g];
        if (degrees) degrees[g] = d;
    }
    std::vector<b2sr_csr_host> gs(count);
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
    for (int g = 0; g < count; ++g) {
        gs[g].rowptr = gs[g].colind = nullptr;
        if (b2sr_graph_er(n[g], m[g], seed * 1000 + (uint64_t)g, &gs[g]) != 0) bad |= 1;
    }
    offsets[0] = 0;
    long long total = 0;
    for (int g = 0; g < count; ++g) {
        total += ((long long)n[g] + align - 1) / align * align;
        if (total > INT_MAX) bad |= 4;
        offsets[g + 1] = (int)total;
    }
    int rc = bad ? (bad & 4 ? 4 : 5) : b2sr_graph_block_diag(gs.data(), offsets, count, out);
    for (auto& h : gs) b2sr_graph_free(&h);
    return rc;
}

int b2sr_graph_block_diag(const b2sr_csr_host* graphs, const int* offsets, int count,
                          b2sr_csr_host* out) {
    if (!out || count < 0 || (count > 0 && (!graphs || !offsets))) return 1;
    long long nnz = 0;
    for (int g = 0; g < count; ++g) {
        if (offsets[g + 1] - offsets[g] < graphs[g].nrows || offsets[g + 1] < offsets[g]) return 1;
        nnz += graphs[g].nnz;
    }
    if (nnz > INT_MAX) return 4;
    const int nrows = count > 0 ? offsets[count] : 0;
    if (!alloc_csr(nrows, nrows, nnz, out)) return 5;
    long long p = 0;
    int row = 0;
    for (int g = 0; g < count; ++g) {
        const b2sr_csr_host& G = graphs[g];
        for (; row < offsets[g]; ++row) out->rowptr[row] = (int)p;
        for (int i = 0; i < G.nrows; ++i, ++row) {
            out->rowptr[row] = (int)p;
            for (int q = G.rowptr[i]; q < G.rowptr[i + 1]; ++q) out->colind[p++] = G.colind[q] + offsets[g];
        }
    }
    for (; row <= nrows; ++row) out->rowptr[row] = (int)p;
    return 0;
}

int b2sr_graph_read_mtx(const char* path, int drop_self_loops, b2sr_csr_host* out) {
    if (!path || !out) return 1;
    FILE* f = std::fopen(path, "r");
    if (!f) return 1;
    char line[1024];
    if (!std::fgets(line, sizeof line, f)) {
        std::fclose(f);
        return 2;
    }
    // Banner: %%MatrixMarket matrix coordinate <field> <symmetry>
    std::string banner(line);
    for (auto& ch : banner) ch = (char)std::tolower((unsigned char)ch);
    if (banner.rfind("%%matrixmarket", 0) != 0 || banner.find("matrix") == std::string::npos ||
        banner.find("coordinate") == std::string::npos || banner.find("complex") != std::string::npos) {
        std::fclose(f);
        return 2;
    }
    const bool pattern = banner.find("pattern") != std::string::npos;
    const bool symmetric = banner.find("symmetric") != std::string::npos ||
                           banner.find("hermitian") != std::string::npos;
    long long M = -1, N = -1, NZ = -1;
    while (std::fgets(line, sizeof line, f)) {
        if (line[0] == '%') continue;
        bool blank = true;
        for (char* q = line; *q; ++q)
            if (!std::isspace((unsigned char)*q)) blank = false;
        if (blank) continue;
        if (std::sscanf(line, "%lld %lld %lld", &M, &N, &NZ) != 3) {
            std::fclose(f);
            return 2;
        }
        break;
    }
    if (M < 0 || N < 0 || NZ < 0 || M > INT_MAX || N > INT_MAX) {
        std::fclose(f);
        return 2;
    }
    std::vector<int> rows((size_t)NZ), cols((size_t)NZ);
    for (long long e = 0; e < NZ; ++e) {
        long long i, j;
        if (std::fscanf(f, "%lld %lld", &i, &j) != 2) {
            std::fclose(f);
            return 3;
        }
        if (!pattern) {
            double val;
            if (std::fscanf(f, "%lf", &val) != 1) {
                std::fclose(f);
                return 3;
            }
        }
        if (i < 1 || i > M || j < 1 || j > N) {
            std::fclose(f);
            return 3;
        }
        rows[(size_t)e] = (int)(i - 1);
        cols[(size_t)e] = (int)(j - 1);
    }
    std::fclose(f);
    if (symmetric && M != N) return 2;
    return b2sr_graph_coo_to_csr(rows.data(), cols.data(), NZ, (int)M, (int)N, symmetric ? 1 : 0,
                                 drop_self_loops, out);
}

}  // extern "C"
