/*
 * A plain-C driver in the shape of the reference's bmv_eval/test_bin_full_full.cu
 * and test_bin_bin_bin.cu, with only the lines that bind those drivers to the
 * reference's packer and kernels changed: the structure pass (cusparseXcsr2bsrNnz, test_bin_full_full.cu:189-190), the
 * packer (csr2bsr_batch_{T}, :196-208), the vector packer (packRandVec /
 * ToBit{T}Row, test_bin_bin_bin.cu:256-281) and the timed kernel launches
 * (evalHSBSFBmv, test_bin_full_full.cu:285-297) call libb2sr instead.
 *
 * It builds a seeded random symmetric graph on the host, multiplies TEST_TIMES
 * times with accumulation (+=, |=) as the reference drivers do, and checks the
 * results against its own host CSR loops: FP32 within 1e-5 of the row's
 * absolute sum, bits exactly.  Then it repeats bin_full_full through the
 * handle API (b2sr_matrix_wrap).  Exit status 0 = all checks passed.
 *
 * usage: drop_in_driver <n> <avg_degree> <tile_dim>
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "b2sr.h"

#define TEST_TIMES 5

#define CHECK_CUDA(x)                                                              \
    do {                                                                           \
        cudaError_t e_ = (x);                                                      \
        if (e_ != cudaSuccess) {                                                   \
            fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_)); \
            return 2;                                                              \
        }                                                                          \
    } while (0)
#define CHECK_B2SR(x)                                                              \
    do {                                                                           \
        b2sr_status s_ = (x);                                                      \
        if (s_ != B2SR_SUCCESS) {                                                  \
            fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, b2sr_status_string(s_)); \
            return 3;                                                              \
        }                                                                          \
    } while (0)

static uint64_t rng_state = 0x243F6A8885A308D3ull;
static uint64_t next_u64(void) {
    rng_state = rng_state * 6364136223846793005ull + 1442695040888963407ull;
    return rng_state >> 11;
}

static int cmp_int(const void* a, const void* b) {
    const int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

int main(int argc, char** argv) {
    if (argc != 4) {
        fprintf(stderr, "usage: %s <n> <avg_degree> <tile_dim>\n", argv[0]);
        return 1;
    }
    const int n = atoi(argv[1]), deg = atoi(argv[2]), T = atoi(argv[3]);
    const int npairs = n * deg / 2;

    /* host CSR: symmetric, no self loops, sorted and de-duplicated rows */
    int* cnt = (int*)calloc((size_t)n + 1, sizeof(int));
    int* eu = (int*)malloc(sizeof(int) * (size_t)npairs);
    int* ev = (int*)malloc(sizeof(int) * (size_t)npairs);
    for (int k = 0; k < npairs; ++k) {
        int u = (int)(next_u64() % (uint64_t)n), v = (int)(next_u64() % (uint64_t)n);
        if (u == v) v = (v + 1) % n;
        eu[k] = u;
        ev[k] = v;
        cnt[u + 1]++;
        cnt[v + 1]++;
    }
    for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    int* col = (int*)malloc(sizeof(int) * (size_t)cnt[n]);
    int* pos = (int*)malloc(sizeof(int) * (size_t)n);
    memcpy(pos, cnt, sizeof(int) * (size_t)n);
    for (int k = 0; k < npairs; ++k) {
        col[pos[eu[k]]++] = ev[k];
        col[pos[ev[k]]++] = eu[k];
    }
    int* rowptr = (int*)malloc(sizeof(int) * ((size_t)n + 1));
    int nnz = 0;
    rowptr[0] = 0;
    for (int i = 0; i < n; ++i) {
        int* r = col + cnt[i];
        const int len = cnt[i + 1] - cnt[i];
        qsort(r, (size_t)len, sizeof(int), cmp_int);
        for (int k = 0; k < len; ++k)
            if (k == 0 || r[k] != r[k - 1]) col[nnz++] = r[k];
        rowptr[i + 1] = nnz;
    }

    /* CSR2HSBSF with the library's structure pass and packer */
    const int nblockrows = (n + T - 1) / T;
    int *csrRowPtr, *csrColInd, *bsrRowPtr, *bsrColInd;
    void* tA;
    int nblocks = 0;
    CHECK_CUDA(cudaMalloc((void**)&csrRowPtr, sizeof(int) * ((size_t)n + 1)));
    CHECK_CUDA(cudaMalloc((void**)&csrColInd, sizeof(int) * (size_t)(nnz > 0 ? nnz : 1)));
    CHECK_CUDA(cudaMemcpy(csrRowPtr, rowptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemcpy(csrColInd, col, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMalloc((void**)&bsrRowPtr, sizeof(int) * ((size_t)nblockrows + 1)));
    CHECK_B2SR(b2sr_ref_csr2bsr_nnz(csrRowPtr, csrColInd, n, n, T, bsrRowPtr, &nblocks));
    const size_t word = T <= 8 ? 1 : (size_t)T / 8;
    CHECK_CUDA(cudaMalloc((void**)&bsrColInd, sizeof(int) * (size_t)(nblocks > 0 ? nblocks : 1)));
    CHECK_CUDA(cudaMalloc(&tA, (size_t)(nblocks > 0 ? nblocks : 1) * T * word));
    CHECK_B2SR(b2sr_ref_csr2bsr_batch(rowptr, col, n, n, nnz, bsrRowPtr, bsrColInd, tA, T, nblockrows, nblocks));

    /* bin_full_full: x ~ U[0,1), y pre-zeroed, TEST_TIMES accumulating launches */
    const size_t npad = (size_t)nblockrows * T;
    float* hx = (float*)calloc(npad, sizeof(float));
    for (int i = 0; i < n; ++i) hx[i] = (float)((next_u64() >> 11) * (1.0 / 9007199254740992.0));
    float *fB, *fC;
    CHECK_CUDA(cudaMalloc((void**)&fB, sizeof(float) * npad));
    CHECK_CUDA(cudaMalloc((void**)&fC, sizeof(float) * npad));
    CHECK_CUDA(cudaMemcpy(fB, hx, sizeof(float) * npad, cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemset(fC, 0, sizeof(float) * npad));
    for (int i = 0; i < TEST_TIMES; i++) CHECK_B2SR(b2sr_ref_bmv_bin_full_full(T, tA, fB, fC, bsrRowPtr, bsrColInd, nblockrows));
    float* hy = (float*)malloc(sizeof(float) * npad);
    CHECK_CUDA(cudaMemcpy(hy, fC, sizeof(float) * npad, cudaMemcpyDeviceToHost));
    double worst = 0.0;
    for (int i = 0; i < n; ++i) {
        double s = 0.0, a = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            s += hx[col[k]];
            a += fabs((double)hx[col[k]]);
        }
        const double err = fabs((double)hy[i] - TEST_TIMES * s) / (TEST_TIMES * a > 0 ? TEST_TIMES * a : 1e-30);
        if (err > worst) worst = err;
    }
    printf("bin_full_full shim: max rel err %.3e over %d rows (%d tiles, T=%d)\n", worst, n, nblocks, T);
    int fail = worst > 1e-5;

    /* bin_bin_bin: frontier bits (x > 0.5), y |= over TEST_TIMES launches */
    float* hf = (float*)calloc(npad, sizeof(float));
    for (int i = 0; i < n; ++i) hf[i] = hx[i] > 0.5f ? 1.0f : 0.0f;
    void *tB, *tC;
    CHECK_CUDA(cudaMalloc(&tB, (size_t)nblockrows * word));
    CHECK_CUDA(cudaMalloc(&tC, (size_t)nblockrows * word));
    CHECK_CUDA(cudaMemcpy(fB, hf, sizeof(float) * npad, cudaMemcpyHostToDevice));
    CHECK_B2SR(b2sr_pack_vec_bits(fB, (int)npad, T, tB, NULL));
    CHECK_CUDA(cudaMemset(tC, 0, (size_t)nblockrows * word));
    for (int i = 0; i < TEST_TIMES; i++) CHECK_B2SR(b2sr_ref_bmv_bin_bin_bin(T, tA, tB, tC, bsrRowPtr, bsrColInd, nblockrows));
    float* hb = (float*)malloc(sizeof(float) * npad);
    CHECK_B2SR(b2sr_unpack_vec_bits(tC, (int)npad, T, fC, NULL));
    CHECK_CUDA(cudaMemcpy(hb, fC, sizeof(float) * npad, cudaMemcpyDeviceToHost));
    int bad = 0;
    for (int i = 0; i < n; ++i) {
        int any = 0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) any |= hf[col[k]] > 0.0f;
        if ((hb[i] > 0.0f) != any) ++bad;
    }
    printf("bin_bin_bin shim: %d wrong rows of %d\n", bad, n);
    fail |= bad != 0;

    /* the handle API on the same arrays (cached plans, row-binned kernel) */
    b2sr_matrix* A = NULL;
    CHECK_CUDA(cudaMemcpy(fB, hx, sizeof(float) * npad, cudaMemcpyHostToDevice));
    CHECK_B2SR(b2sr_matrix_wrap(bsrRowPtr, bsrColInd, tA, n, n, nblocks, T, NULL, &A));
    CHECK_B2SR(b2sr_spmv_bin_full_full(A, fB, fC, 0, NULL));
    CHECK_CUDA(cudaMemcpy(hy, fC, sizeof(float) * npad, cudaMemcpyDeviceToHost));
    worst = 0.0;
    for (int i = 0; i < n; ++i) {
        double s = 0.0, a = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            s += hx[col[k]];
            a += fabs((double)hx[col[k]]);
        }
        const double err = fabs((double)hy[i] - s) / (a > 0 ? a : 1e-30);
        if (err > worst) worst = err;
    }
    printf("bin_full_full handle: max rel err %.3e\n", worst);
    fail |= worst > 1e-5;
    b2sr_free(A);

    cudaFree(csrRowPtr);
    cudaFree(csrColInd);
    cudaFree(bsrRowPtr);
    cudaFree(bsrColInd);
    cudaFree(tA);
    cudaFree(fB);
    cudaFree(fC);
    cudaFree(tB);
    cudaFree(tC);
    free(cnt);
    free(eu);
    free(ev);
    free(col);
    free(pos);
    free(rowptr);
    free(hx);
    free(hy);
    free(hf);
    free(hb);
    printf(fail ? "FAILED\n" : "PASSED\n");
    return fail ? 4 : 0;
}
