/*
 * CPU oracle of the B2SR binary SpMV path — TEST INFRASTRUCTURE ONLY (the
 * checker of the tests, the smoke check and the CPU baseline of the
 * benchmark; the library never links or calls it).  Plain C99 + OpenMP.
 *
 * The restated reference code lives in hsung2/Bit-GraphBLAS under bmv_eval/;
 * each function cites the lines it follows.
 */
#include "b2sr_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static uint32_t get_word(const void* w, long long i, int T) {
    if (T <= 8) return ((const uint8_t*)w)[i];
    if (T == 16) return ((const uint16_t*)w)[i];
    return ((const uint32_t*)w)[i];
}

static void put_word(void* w, long long i, int T, uint32_t v) {
    if (T <= 8) ((uint8_t*)w)[i] = (uint8_t)v;
    else if (T == 16) ((uint16_t*)w)[i] = (uint16_t)v;
    else ((uint32_t*)w)[i] = v;
}

static int popc32(uint32_t v) {
    int c = 0;
    while (v) {
        v &= v - 1;
        ++c;
    }
    return c;
}

static int cmp_int(const void* a, const void* b) {
    const int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

/* Distinct tile-columns per tile-row: what cusparseXcsr2bsrNnz computes
 * (bmv_eval/test_bin_full_full.cu:189-190). */
long long oracle_b2sr_structure(const int* rowptr, const int* colind, int nrows, int T,
                                int* browptr) {
    const int nb = (nrows + T - 1) / T;
    int max_col = -1;
    for (long long p = 0; p < rowptr[nrows]; ++p)
        if (colind[p] > max_col) max_col = colind[p];
    const int nbc = max_col / T + 1;
    int* seen = (int*)calloc((size_t)nbc + 1, sizeof(int));
    long long nt = 0;
    browptr[0] = 0;
    for (int tr = 0; tr < nb; ++tr) {
        for (int r = tr * T; r < (tr + 1) * T && r < nrows; ++r)
            for (int p = rowptr[r]; p < rowptr[r + 1]; ++p) {
                const int bc = colind[p] / T;
                if (seen[bc] != tr + 1) {
                    seen[bc] = tr + 1;
                    ++nt;
                }
            }
        browptr[tr + 1] = (int)nt;
    }
    free(seen);
    return nt;
}

/* Tiles of each tile-row in ascending tile-column order, as cusparseScsr2bsr
 * with CUSPARSE_DIRECTION_ROW emits them (bmv_eval/backend/csr2bsr_batch_bsrbmv.cu:61,100),
 * bit-packed as ToBit{T}Col does: row r of the dense tile becomes word r with
 * column c at bit T-1-c (bmv_eval/backend/bsrbmv.cu:33-62 for T = 4, :92-114 for 8,
 * :139-159 for 16, :186-203 for 32). */
void oracle_b2sr_fill(const int* rowptr, const int* colind, int nrows, int T, const int* browptr,
                      int* bcolind, void* tiles) {
    const int nb = (nrows + T - 1) / T;
    int max_col = -1;
    for (long long p = 0; p < rowptr[nrows]; ++p)
        if (colind[p] > max_col) max_col = colind[p];
    const int nbc = max_col / T + 1;
    int* slot = (int*)malloc(((size_t)nbc + 1) * sizeof(int));
    for (int i = 0; i <= nbc; ++i) slot[i] = -1;
    memset(tiles, 0, (size_t)browptr[nb] * T * (T <= 8 ? 1 : T / 8));
    for (int tr = 0; tr < nb; ++tr) {
        const int b = browptr[tr], e = browptr[tr + 1];
        int n = 0;
        for (int r = tr * T; r < (tr + 1) * T && r < nrows; ++r)
            for (int p = rowptr[r]; p < rowptr[r + 1]; ++p) {
                const int bc = colind[p] / T;
                if (slot[bc] != -2) {
                    slot[bc] = -2;
                    bcolind[b + n++] = bc;
                }
            }
        qsort(bcolind + b, (size_t)(e - b), sizeof(int), cmp_int);
        for (int k = b; k < e; ++k) slot[bcolind[k]] = k;
        for (int r = tr * T; r < (tr + 1) * T && r < nrows; ++r)
            for (int p = rowptr[r]; p < rowptr[r + 1]; ++p) {
                const int c = colind[p];
                const long long w = (long long)slot[c / T] * T + (r - tr * T);
                put_word(tiles, w, T, get_word(tiles, w, T) | (1u << (T - 1 - c % T)));
            }
        for (int k = b; k < e; ++k) slot[bcolind[k]] = -1;
    }
    free(slot);
}

/* ToBit{T}Row (bmv_eval/backend/bsrbmv.cu:64-90, 116-137, 162-181, 205-222): each
 * word collects (x > 0) of T consecutive elements, the first at the MSB. */
void oracle_pack_vec_bits(const float* x, int n, int T, void* bits) {
    const int nw = (n + T - 1) / T;
    for (int j = 0; j < nw; ++j) {
        uint32_t w = 0;
        for (int c = 0; c < T; ++c) {
            const long long i = (long long)j * T + c;
            w = (w << 1) | (uint32_t)(i < n && x[i] > 0.0f);
        }
        put_word(bits, j, T, w);
    }
}

/* bin2full (bmv_eval/backend/utility.cu:156-178). */
void oracle_unpack_vec_bits(const void* bits, int n, int T, float* out) {
    for (int i = 0; i < n; ++i) {
        const uint32_t w = get_word(bits, i / T, T);
        out[i] = ((w >> (T - 1 - i % T)) & 1u) ? 1.0f : 0.0f;
    }
}

/* bmv{4,8,16,32}_bin_bin_bin (bmv_eval/backend/bsrbmv.cu:277-310, 437-470, 508-541,
 * 579-613): per tile row, Cm += popc(A_row & x[colind]); the output bit is
 * Cm > 0, MSB = row 0, OR-ed into y. */
static uint32_t bin_bin_bin_row(int T, const int* rowptr, const int* colind, const void* tiles,
                                const void* xbits, int i) {
    uint32_t out = 0;
    for (int r = 0; r < T; ++r) {
        int cm = 0;
        for (int t = rowptr[i]; t < rowptr[i + 1]; ++t)
            cm += popc32(get_word(tiles, (long long)t * T + r, T) & get_word(xbits, colind[t], T));
        if (cm > 0) out |= 1u << (T - 1 - r);
    }
    return out;
}

void oracle_bmv_bin_bin_bin(int T, int nb, const int* rowptr, const int* colind, const void* tiles,
                            const void* xbits, void* ybits, int accumulate) {
    for (int i = 0; i < nb; ++i) {
        uint32_t v = bin_bin_bin_row(T, rowptr, colind, tiles, xbits, i);
        if (accumulate) v |= get_word(ybits, i, T);
        put_word(ybits, i, T, v);
    }
}

/* bmv{T}_bin_bin_bin_masked (bmv_eval/backend/bsrbmv.cu:1086-1229): the result ANDed
 * with ~mask[row], overwriting y.  The T = 8 and 16 kernels there shift by
 * 32 - ... and keep only 4 bits (bsrbmv.cu:1153, 1189); the oracle states the
 * intended full-width mask. */
void oracle_bmv_bin_bin_bin_masked(int T, int nb, const int* rowptr, const int* colind,
                                   const void* tiles, const void* xbits, const void* maskbits,
                                   void* ybits) {
    const uint32_t full = T == 32 ? 0xffffffffu : ((1u << T) - 1u);
    for (int i = 0; i < nb; ++i) {
        const uint32_t v = bin_bin_bin_row(T, rowptr, colind, tiles, xbits, i);
        put_word(ybits, i, T, v & ~get_word(maskbits, i, T) & full);
    }
}

/* bmv{4,8,16,32}_bin_bin_full (bmv_eval/backend/bsrbmv.cu:618-676, 678-736, 738-787,
 * 789-821): y[i*T + r] += popc(A_row_r & x[colind]) summed over the tile-row. */
void oracle_bmv_bin_bin_count(int T, int nb, const int* rowptr, const int* colind,
                              const void* tiles, const void* xbits, int* y, int accumulate) {
    for (int i = 0; i < nb; ++i)
        for (int r = 0; r < T; ++r) {
            int cm = 0;
            for (int t = rowptr[i]; t < rowptr[i + 1]; ++t)
                cm += popc32(get_word(tiles, (long long)t * T + r, T) & get_word(xbits, colind[t], T));
            y[(long long)i * T + r] = accumulate ? y[(long long)i * T + r] + cm : cm;
        }
}

void oracle_bmv_bin_bin_full(int T, int nb, const int* rowptr, const int* colind, const void* tiles,
                             const void* xbits, float* y, int accumulate) {
    for (int i = 0; i < nb; ++i)
        for (int r = 0; r < T; ++r) {
            int cm = 0;
            for (int t = rowptr[i]; t < rowptr[i + 1]; ++t)
                cm += popc32(get_word(tiles, (long long)t * T + r, T) & get_word(xbits, colind[t], T));
            y[(long long)i * T + r] = accumulate ? y[(long long)i * T + r] + (float)cm : (float)cm;
        }
}

/* bmv32_bin_full_full (bmv_eval/backend/bsrbmv.cu:1040-1081): for each tile in colind
 * order, for j = 0..T-1, sum += x[colind*T + j] when bit T-1-j of the row is
 * set; then y += sum. */
void oracle_bmv_bin_full_full(int T, int nb, const int* rowptr, const int* colind,
                              const void* tiles, const float* x, float* y, int accumulate) {
    for (int i = 0; i < nb; ++i)
        for (int r = 0; r < T; ++r) {
            float sum = 0.0f;
            for (int t = rowptr[i]; t < rowptr[i + 1]; ++t) {
                const uint32_t w = get_word(tiles, (long long)t * T + r, T);
                for (int j = 0; j < T; ++j)
                    if ((w >> (T - 1 - j)) & 1u) sum += x[(long long)colind[t] * T + j];
            }
            y[(long long)i * T + r] = accumulate ? y[(long long)i * T + r] + sum : sum;
        }
}

void oracle_bmv_bin_full_full_f64(int T, int nb, const int* rowptr, const int* colind,
                                  const void* tiles, const float* x, double* y) {
    for (int i = 0; i < nb; ++i)
        for (int r = 0; r < T; ++r) {
            double sum = 0.0;
            for (int t = rowptr[i]; t < rowptr[i + 1]; ++t) {
                const uint32_t w = get_word(tiles, (long long)t * T + r, T);
                for (int j = 0; j < T; ++j)
                    if ((w >> (T - 1 - j)) & 1u) sum += (double)x[(long long)colind[t] * T + j];
            }
            y[(long long)i * T + r] = sum;
        }
}

void oracle_bmm_f64(int T, int nb, const int* rowptr, const int* colind, const void* tiles,
                    const double* X, int k, int ldx, double* Y, int ldy) {
    for (int i = 0; i < nb; ++i)
        for (int r = 0; r < T; ++r) {
            double* yr = Y + ((long long)i * T + r) * ldy;
            for (int q = 0; q < k; ++q) yr[q] = 0.0;
            for (int t = rowptr[i]; t < rowptr[i + 1]; ++t) {
                const uint32_t w = get_word(tiles, (long long)t * T + r, T);
                for (int j = 0; j < T; ++j)
                    if ((w >> (T - 1 - j)) & 1u) {
                        const double* xr = X + ((long long)colind[t] * T + j) * ldx;
                        for (int q = 0; q < k; ++q) yr[q] += xr[q];
                    }
            }
        }
}

/* The reference's correctness check multiplies the CSR with all values forced
 * to 1 (setDeviceValArr, bmv_eval/test_bin_full_full.cu:155) by cuSPARSE csrmv
 * (bmv_eval/test_bin_full_full.cu:262); here in FP64. */
void oracle_csr_spmv_f64(const int* rowptr, const int* colind, int nrows, const float* x,
                         double* y) {
    for (int i = 0; i < nrows; ++i) {
        double s = 0.0;
        for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) s += (double)x[colind[p]];
        y[i] = s;
    }
}

void oracle_csr_spmv_abs_f64(const int* rowptr, const int* colind, int nrows, const float* x,
                             double* y) {
    for (int i = 0; i < nrows; ++i) {
        double s = 0.0;
        for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) {
            const double v = (double)x[colind[p]];
            s += v < 0 ? -v : v;
        }
        y[i] = s;
    }
}

void oracle_csr_spmv_count(const int* rowptr, const int* colind, int nrows, const uint8_t* xb,
                           long long* y) {
    for (int i = 0; i < nrows; ++i) {
        long long s = 0;
        for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) s += xb[colind[p]] != 0;
        y[i] = s;
    }
}

int oracle_csr_spmv_f32_omp(const int* rowptr, const int* colind, int nrows, const float* x,
                            float* y, int nthreads) {
    int used = 1;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
    {
#pragma omp single
        used = omp_get_num_threads();
#pragma omp for schedule(static)
        for (int i = 0; i < nrows; ++i) {
            float s = 0.0f;
            for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) s += x[colind[p]];
            y[i] = s;
        }
    }
#else
    (void)nthreads;
    for (int i = 0; i < nrows; ++i) {
        float s = 0.0f;
        for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) s += x[colind[p]];
        y[i] = s;
    }
#endif
    return used;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---- inputs of the benchmark's CPU arm ---- */
static uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void oracle_rmat_edges(int scale, long long m, double a, double b, double c, uint64_t seed, int* u,
                       int* v) {
    const uint64_t key = mix64(seed ^ 0x5851F42D4C957F2Dull);
    const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
    for (long long e = 0; e < m; ++e) {
        int uu = 0, vv = 0;
        for (int l = 0; l < scale; ++l) {
            const uint64_t z = mix64(key + ((uint64_t)e * (uint64_t)scale + (uint64_t)l) * 0xD1B54A32D192ED03ull);
            const double r = (double)(z >> 11) * (1.0 / 9007199254740992.0);
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
        u[e] = uu;
        v[e] = vv;
    }
}

long long oracle_sym_csr(const int* u, const int* v, long long m, int n, int* rowptr, int* colind) {
    long long* off = (long long*)calloc((size_t)n + 1, sizeof(long long));
    long long* kept = (long long*)calloc((size_t)n + 1, sizeof(long long));
    if (!off || !kept) {
        free(off);
        free(kept);
        return -1;
    }
    for (long long e = 0; e < m; ++e)
        if (u[e] != v[e]) {
            off[u[e] + 1]++;
            off[v[e] + 1]++;
        }
    for (int i = 0; i < n; ++i) off[i + 1] += off[i];
    {
        long long* pos = (long long*)malloc(sizeof(long long) * ((size_t)n + 1));
        if (!pos) {
            free(off);
            free(kept);
            return -1;
        }
        memcpy(pos, off, sizeof(long long) * ((size_t)n + 1));
        for (long long e = 0; e < m; ++e)
            if (u[e] != v[e]) {
                colind[pos[u[e]]++] = v[e];
                colind[pos[v[e]]++] = u[e];
            }
        free(pos);
    }
#pragma omp parallel for schedule(dynamic, 1024)
    for (int i = 0; i < n; ++i) {
        int* r = colind + off[i];
        const long long len = off[i + 1] - off[i];
        if (len > 1) qsort(r, (size_t)len, sizeof(int), cmp_int);
        long long k = 0;
        for (long long j = 0; j < len; ++j)
            if (k == 0 || r[j] != r[k - 1]) r[k++] = r[j];
        kept[i + 1] = k;
    }
    for (int i = 0; i < n; ++i) kept[i + 1] += kept[i];
    const long long nnz = kept[n];
    if (nnz <= 2147483647LL) {
        /* rows only move towards the front: kept[i] <= off[i] */
        for (int i = 0; i < n; ++i) {
            const long long len = kept[i + 1] - kept[i];
            if (len && kept[i] != off[i]) memmove(colind + kept[i], colind + off[i], sizeof(int) * (size_t)len);
            rowptr[i] = (int)kept[i];
        }
        rowptr[n] = (int)nnz;
    }
    free(off);
    free(kept);
    return nnz <= 2147483647LL ? nnz : -1;
}
