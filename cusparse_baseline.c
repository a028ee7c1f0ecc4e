/*
 * cuSPARSE baselines of the benchmark (bench.py), called through ctypes: the
 * reference's own comparison target, evalCSRSpmvFloatCuSPARSE
 * (bmv_eval/test_spmv_baseline_a100.cu:92-146, bmv_eval/test_bin_full_full.cu:233-272),
 * re-expressed with the generic API because CUDA 13 removed cusparseScsrmv and
 * CUSPARSE_CSRMV_ALG1: cusparseSpMV over a CSR matrix with all values 1, FP32,
 * with an explicit algorithm (CUSPARSE_SPMV_CSR_ALG1 as the reference names,
 * or ALG2), and cusparseSpMM for dense right-hand sides.  Compiled by bench.py
 * with gcc and linked against the toolkit's libcusparse only; the B2SR
 * library never loads it.
 */
#include <cuda_runtime.h>
#include <cusparse.h>
#include <stdlib.h>

typedef struct {
    cusparseHandle_t handle;
    cusparseSpMatDescr_t mat;
    int nrows, ncols;
    float* vals;
    void* buffer;
    size_t buffer_bytes;
} cus_csr;

void cus_csr_destroy(void* h);

/* 0 on success; a negative value names the failing step (nothing is kept then). */
int cus_csr_create(int nrows, int ncols, int nnz, const int* d_rowptr, const int* d_colind, void** out) {
    cus_csr* c = (cus_csr*)calloc(1, sizeof(cus_csr));
    float* h = NULL;
    int rc = 0;
    *out = NULL;
    if (!c) return -1;
    c->nrows = nrows;
    c->ncols = ncols;
    if (cudaMalloc((void**)&c->vals, sizeof(float) * (size_t)(nnz > 0 ? nnz : 1)) != cudaSuccess) {
        c->vals = NULL;
        rc = -2;
        goto fail;
    }
    /* values 1: filled through a host staging copy (setup, not timed) */
    h = (float*)malloc(sizeof(float) * (size_t)(nnz > 0 ? nnz : 1));
    if (!h) {
        rc = -3;
        goto fail;
    }
    for (int i = 0; i < nnz; ++i) h[i] = 1.0f;
    if (cudaMemcpy(c->vals, h, sizeof(float) * (size_t)nnz, cudaMemcpyHostToDevice) != cudaSuccess) {
        rc = -4;
        goto fail;
    }
    if (cusparseCreate(&c->handle) != CUSPARSE_STATUS_SUCCESS) {
        c->handle = NULL;
        rc = -5;
        goto fail;
    }
    if (cusparseCreateCsr(&c->mat, nrows, ncols, nnz, (void*)d_rowptr, (void*)d_colind, c->vals,
                          CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I, CUSPARSE_INDEX_BASE_ZERO,
                          CUDA_R_32F) != CUSPARSE_STATUS_SUCCESS) {
        c->mat = NULL;
        rc = -6;
        goto fail;
    }
    free(h);
    *out = c;
    return 0;
fail:
    free(h);
    cus_csr_destroy(c);
    return rc;
}

static int ensure_buffer(cus_csr* c, size_t bytes) {
    if (bytes <= c->buffer_bytes) return 0;
    if (c->buffer) cudaFree(c->buffer);
    c->buffer = NULL;
    c->buffer_bytes = 0;
    if (cudaMalloc(&c->buffer, bytes ? bytes : 16) != cudaSuccess) return -1;
    c->buffer_bytes = bytes;
    return 0;
}

/* y = A.x + beta*y with the given cusparseSpMVAlg_t (1 = CUSPARSE_SPMV_CSR_ALG1,
 * 2 = CUSPARSE_SPMV_CSR_ALG2).  prepare != 0 sizes the work buffer and runs
 * cusparseSpMV_preprocess (setup, outside any timed region). */
int cus_spmv(void* h, int alg, const float* d_x, float* d_y, float beta, int prepare, void* stream) {
    cus_csr* c = (cus_csr*)h;
    const cusparseSpMVAlg_t a = alg == 2 ? CUSPARSE_SPMV_CSR_ALG2 : CUSPARSE_SPMV_CSR_ALG1;
    cusparseDnVecDescr_t x, y;
    const float alpha = 1.0f;
    int rc = 0;
    if (cusparseSetStream(c->handle, (cudaStream_t)stream) != CUSPARSE_STATUS_SUCCESS) return -1;
    if (cusparseCreateDnVec(&x, c->ncols, (void*)d_x, CUDA_R_32F) != CUSPARSE_STATUS_SUCCESS) return -2;
    if (cusparseCreateDnVec(&y, c->nrows, d_y, CUDA_R_32F) != CUSPARSE_STATUS_SUCCESS) return -3;
    if (prepare) {
        size_t bytes = 0;
        if (cusparseSpMV_bufferSize(c->handle, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, c->mat, x, &beta, y,
                                    CUDA_R_32F, a, &bytes) != CUSPARSE_STATUS_SUCCESS)
            rc = -4;
        else if (ensure_buffer(c, bytes) != 0)
            rc = -5;
        else if (cusparseSpMV_preprocess(c->handle, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, c->mat, x, &beta, y,
                                         CUDA_R_32F, a, c->buffer) != CUSPARSE_STATUS_SUCCESS)
            rc = -6;
    }
    if (rc == 0 && cusparseSpMV(c->handle, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, c->mat, x, &beta, y,
                                CUDA_R_32F, a, c->buffer) != CUSPARSE_STATUS_SUCCESS)
        rc = -7;
    cusparseDestroyDnVec(x);
    cusparseDestroyDnVec(y);
    return rc;
}

/* Y = op(A).X (row-major X [rows_x, k], Y [rows_y, k]) with CUSPARSE_SPMM_CSR_ALG2;
 * transpose != 0 multiplies by A^T (the adjoint). */
int cus_spmm(void* h, int transpose, const float* d_X, int k, float* d_Y, int prepare, void* stream) {
    cus_csr* c = (cus_csr*)h;
    const cusparseOperation_t op = transpose ? CUSPARSE_OPERATION_TRANSPOSE : CUSPARSE_OPERATION_NON_TRANSPOSE;
    const int rx = transpose ? c->nrows : c->ncols, ry = transpose ? c->ncols : c->nrows;
    cusparseDnMatDescr_t X, Y;
    const float alpha = 1.0f, beta = 0.0f;
    int rc = 0;
    if (cusparseSetStream(c->handle, (cudaStream_t)stream) != CUSPARSE_STATUS_SUCCESS) return -1;
    if (cusparseCreateDnMat(&X, rx, k, k, (void*)d_X, CUDA_R_32F, CUSPARSE_ORDER_ROW) != CUSPARSE_STATUS_SUCCESS)
        return -2;
    if (cusparseCreateDnMat(&Y, ry, k, k, d_Y, CUDA_R_32F, CUSPARSE_ORDER_ROW) != CUSPARSE_STATUS_SUCCESS) return -3;
    if (prepare) {
        size_t bytes = 0;
        if (cusparseSpMM_bufferSize(c->handle, op, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, c->mat, X, &beta, Y,
                                    CUDA_R_32F, CUSPARSE_SPMM_CSR_ALG2, &bytes) != CUSPARSE_STATUS_SUCCESS)
            rc = -4;
        else if (ensure_buffer(c, bytes) != 0)
            rc = -5;
        else if (cusparseSpMM_preprocess(c->handle, op, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, c->mat, X, &beta,
                                         Y, CUDA_R_32F, CUSPARSE_SPMM_CSR_ALG2, c->buffer) != CUSPARSE_STATUS_SUCCESS)
            rc = -6;
    }
    if (rc == 0 && cusparseSpMM(c->handle, op, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, c->mat, X, &beta, Y,
                                CUDA_R_32F, CUSPARSE_SPMM_CSR_ALG2, c->buffer) != CUSPARSE_STATUS_SUCCESS)
        rc = -7;
    cusparseDestroyDnMat(X);
    cusparseDestroyDnMat(Y);
    return rc;
}

void cus_csr_destroy(void* h) {
    cus_csr* c = (cus_csr*)h;
    if (!c) return;
    cudaDeviceSynchronize();
    if (c->mat) cusparseDestroySpMat(c->mat);
    if (c->handle) cusparseDestroy(c->handle);
    if (c->buffer) cudaFree(c->buffer);
    if (c->vals) cudaFree(c->vals);
    free(c);
}
