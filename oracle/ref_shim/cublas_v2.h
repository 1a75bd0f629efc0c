/* cuBLAS stand-in for the CPU build of the reference (TEST INFRASTRUCTURE ONLY).
 * Textbook summation order, identical to the oracle's dense routines. */
#ifndef SA_CUBLAS_V2_H
#define SA_CUBLAS_V2_H
#include <cstddef>
typedef struct sa_blas_handle *cublasHandle_t;
typedef int cublasStatus_t;
typedef enum { CUBLAS_OP_N = 0, CUBLAS_OP_T = 1 } cublasOperation_t;
typedef enum { CUBLAS_FILL_MODE_LOWER = 0, CUBLAS_FILL_MODE_UPPER = 1 } cublasFillMode_t;
cublasStatus_t cublasCreate(cublasHandle_t *h);
cublasStatus_t cublasDestroy(cublasHandle_t h);
cublasStatus_t cublasDdot(cublasHandle_t h, int n, const double *x, int incx, const double *y, int incy,
                          double *result);
cublasStatus_t cublasDgemv(cublasHandle_t h, cublasOperation_t t, int m, int n, const double *alpha,
                           const double *A, int lda, const double *x, int incx, const double *beta,
                           double *y, int incy);
cublasStatus_t cublasDgemm(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                           const double *alpha, const double *A, int lda, const double *B, int ldb,
                           const double *beta, double *C, int ldc);
#endif
