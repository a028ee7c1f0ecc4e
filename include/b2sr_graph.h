/*
 * b2sr_graph.h — host-side graph ingest for the B2SR library: the canonical
 * CSR the reference builds from a Matrix Market file, and seeded synthetic
 * graphs in the same form.
 *
 * Canonical form (bmv_eval/backend/readMtx.hpp:152-218 removeSelfloop and
 * :248-306 coo2csr): optionally mirrored edges, self-loops removed, duplicates
 * removed, rows sorted by column.  All values are 1.
 *
 * Arrays returned through int** / long long* out-parameters are allocated by
 * the library with malloc and released with b2sr_graph_free.
 */
#ifndef B2SR_GRAPH_H_
#define B2SR_GRAPH_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nrows, ncols;
    long long nnz;
    int* rowptr;   /* nrows + 1 */
    int* colind;   /* nnz */
} b2sr_csr_host;

/* 0 on success, nonzero on error (bad arguments, allocation failure, int32 overflow). */

/* COO edge list -> canonical CSR.  symmetrize != 0 adds (v, u) for every
 * (u, v); drop_self_loops != 0 removes (u, u).  Duplicates are always merged. */
int b2sr_graph_coo_to_csr(const int* rows, const int* cols, long long nedges, int nrows, int ncols,
                          int symmetrize, int drop_self_loops, b2sr_csr_host* out);

/* R-MAT graph: 2^scale vertices, edge_factor * 2^scale generated edges, quadrant
 * probabilities (a, b, c, 1-a-b-c), no noise and no vertex permutation, then
 * symmetrised, self-loops and duplicates removed.  Deterministic in `seed`
 * and independent of the thread count. */
int b2sr_graph_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed,
                    b2sr_csr_host* out);

/* Erdos-Renyi graph with exactly m distinct unordered pairs {u, v}, u != v,
 * drawn uniformly, mirrored (nnz = 2m).  Requires m <= n(n-1)/2. */
int b2sr_graph_er(int n, long long m, uint64_t seed, b2sr_csr_host* out);

/* Block-diagonal stack of graphs: vertex ranges of graph g start at offsets[g]
 * (ascending, offsets[count] = total rows); returns the stacked CSR. */
int b2sr_graph_block_diag(const b2sr_csr_host* graphs, const int* offsets, int count,
                          b2sr_csr_host* out);

/* `count` Erdos-Renyi graphs stacked block-diagonally (the uneven-batch
 * workload): graph g has n_g = round(exp(U[ln n_min, ln n_max])) vertices and
 * average degree d_g ~ U[deg_min, deg_max] (m_g = round(n_g d_g / 2) pairs,
 * seed*1000 + g), and its vertex range starts at offsets[g], a multiple of
 * `align` (so no T x T tile with T | align straddles two graphs).  offsets
 * has count + 1 entries; sizes (count) and degrees (count) may be NULL.
 * Graphs are generated in parallel. */
int b2sr_graph_er_batch(int count, double n_min, double n_max, double deg_min, double deg_max, int align,
                        uint64_t seed, b2sr_csr_host* out, int* offsets, int* sizes, double* degrees);

/* Matrix Market coordinate file -> canonical CSR as readMtx does with
 * directed = 0 (bmv_eval/backend/readMtx.hpp:354-422): a "symmetric" banner mirrors
 * the entries; self-loops are removed unless drop_self_loops == 0; pattern,
 * integer and real files are accepted and every value becomes 1.
 * Returns 0, or 1 for a missing file, 2 for a bad banner/size line, 3 for
 * missing entries or out-of-range indices. */
int b2sr_graph_read_mtx(const char* path, int drop_self_loops, b2sr_csr_host* out);

/* Uniform doubles of the generators' counter-based stream (for tests that
 * re-derive sampled values): out[i] = U(seed, first + i). */
void b2sr_graph_uniform(uint64_t seed, long long first, long long count, double* out);

void b2sr_graph_free(b2sr_csr_host* g);

#ifdef __cplusplus
}
#endif

#endif
