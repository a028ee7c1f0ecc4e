/*
 * b2sr_oracle.h — CPU oracle of the B2SR binary SpMV path.  TEST
 * INFRASTRUCTURE ONLY: the tests, the smoke check and the benchmark's CPU
 * baseline use it as the checker; the library never links or calls it.
 *
 * Every function restates the reference's algorithm on the host, citing the
 * reference file:line it follows (paths inside hsung2/Bit-GraphBLAS).
 * Word layout (all tile sizes): word r of a tile holds tile row r, bit (T-1-c)
 * is column c; uint8 words for T = 4 (low nibble) and 8, uint16 for 16, uint32
 * for 32.
 */
#ifndef B2SR_ORACLE_H_
#define B2SR_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* CSR -> B2SR structure: browptr[nb+1]; returns nt.  Follows
 * cusparseXcsr2bsrNnz as called in CSR2HSBSF (bmv_eval/test_bin_full_full.cu:167-211):
 * a tile exists when any entry of its T x T block exists. */
long long oracle_b2sr_structure(const int* rowptr, const int* colind, int nrows, int T,
                                int* browptr);
/* CSR -> B2SR tiles: tile-columns ascending within a tile-row (cusparseScsr2bsr,
 * bmv_eval/backend/csr2bsr_batch_bsrbmv.cu:100), bit rows as ToBit{T}Col
 * (bmv_eval/backend/bsrbmv.cu:33-203).  tiles must hold nt*T words and is overwritten. */
void oracle_b2sr_fill(const int* rowptr, const int* colind, int nrows, int T, const int* browptr,
                      int* bcolind, void* tiles);

/* x[j*T + c] > 0 -> bit (T-1-c) of word j (ToBit{T}Row, bmv_eval/backend/bsrbmv.cu:64-222);
 * writes ceil(n/T) words. */
void oracle_pack_vec_bits(const float* x, int n, int T, void* bits);
/* bin2full (bmv_eval/backend/utility.cu:156-178): bit i -> 1.0f / 0.0f. */
void oracle_unpack_vec_bits(const void* bits, int n, int T, float* out);

/* ---- multiplies on B2SR, restating the reference kernels' arithmetic ---- */
/* bmv{T}_bin_bin_bin (bmv_eval/backend/bsrbmv.cu:277-613): y bit r of tile-row i is set
 * when popc(A_row_r & x_word) > 0 for any tile; OR-accumulates when accumulate. */
void oracle_bmv_bin_bin_bin(int T, int nb, const int* rowptr, const int* colind, const void* tiles,
                            const void* xbits, void* ybits, int accumulate);
/* Masked form (bmv_eval/backend/bsrbmv.cu:1086-1229, intended semantics): y = result & ~mask. */
void oracle_bmv_bin_bin_bin_masked(int T, int nb, const int* rowptr, const int* colind,
                                   const void* tiles, const void* xbits, const void* maskbits,
                                   void* ybits);
/* bmv{T}_bin_bin_full (bmv_eval/backend/bsrbmv.cu:618-821): y[i*T + r] += sum of popc. */
void oracle_bmv_bin_bin_full(int T, int nb, const int* rowptr, const int* colind, const void* tiles,
                             const void* xbits, float* y, int accumulate);
void oracle_bmv_bin_bin_count(int T, int nb, const int* rowptr, const int* colind,
                              const void* tiles, const void* xbits, int* y, int accumulate);
/* bmv{T}_bin_full_full (bmv_eval/backend/bsrbmv.cu:826-1081) in the order of the
 * deterministic T = 32 kernel (bsrbmv.cu:1063-1076): tiles in colind order,
 * columns ascending, FP32. */
void oracle_bmv_bin_full_full(int T, int nb, const int* rowptr, const int* colind,
                              const void* tiles, const float* x, float* y, int accumulate);
/* The same sum in FP64 (the accuracy reference). */
void oracle_bmv_bin_full_full_f64(int T, int nb, const int* rowptr, const int* colind,
                                  const void* tiles, const float* x, double* y);
/* SpMM form: Y[i*T + r, :] = sum over set bits (r, c) of X[tc*T + c, :]; X has
 * ncols rows of k doubles (row stride ldx), Y nb*T rows (row stride ldy). */
void oracle_bmm_f64(int T, int nb, const int* rowptr, const int* colind, const void* tiles,
                    const double* X, int k, int ldx, double* Y, int ldy);

/* ---- CSR oracle, independent of any packing (the reference's cuSPARSE check,
 * bmv_eval/test_bin_full_full.cu:233-272, with all values forced to 1) ---- */
void oracle_csr_spmv_f64(const int* rowptr, const int* colind, int nrows, const float* x,
                         double* y);
/* sum_j |x_j| per row: the scale of the accuracy bound. */
void oracle_csr_spmv_abs_f64(const int* rowptr, const int* colind, int nrows, const float* x,
                             double* y);
/* counts of neighbours j with xb[j] != 0 (xb: one byte per element). */
void oracle_csr_spmv_count(const int* rowptr, const int* colind, int nrows, const uint8_t* xb,
                           long long* y);

/* The timed CPU baseline: FP32 CSR SpMV, values 1, OpenMP over rows (static
 * schedule).  Returns the number of threads used. */
int oracle_csr_spmv_f32_omp(const int* rowptr, const int* colind, int nrows, const float* x,
                            float* y, int nthreads);
int oracle_max_threads(void);

/* ---- inputs of the benchmark's CPU arm ---- */
/* Edge list of the seeded R-MAT generator the library's b2sr_graph_rmat
 * uses (include/b2sr_graph.h), restated so that the CPU arm builds the same
 * graph without loading the library: edge e descends `scale` levels of the
 * adjacency quadtree, level l taking counter-based draw e*scale + l of the
 * splitmix64 stream of `seed` (Steele, Lea & Flood, OOPSLA 2014) and picking
 * quadrant (0,0) below a, (0,1) below a+b, (1,0) below a+b+c, else (1,1).
 * Writes m (u, v) pairs, unsymmetrised and with self-loops and duplicates. */
void oracle_rmat_edges(int scale, long long m, double a, double b, double c, uint64_t seed, int* u,
                       int* v);
/* Canonical symmetric CSR of an edge list (the form readMtx builds,
 * bmv_eval/backend/readMtx.hpp:152-218 removeSelfloop and :248-306 coo2csr):
 * (u, v) and (v, u) for every edge, self-loops dropped, each row sorted and
 * de-duplicated.  rowptr has n + 1 entries; colind must hold 2m entries and
 * receives the nnz kept.  Returns nnz, or -1 if it exceeds the int32 range. */
long long oracle_sym_csr(const int* u, const int* v, long long m, int n, int* rowptr, int* colind);

#ifdef __cplusplus
}
#endif

#endif
