/* cuSOLVER stand-in for the CPU build of the reference (TEST INFRASTRUCTURE ONLY). */
#ifndef SA_CUSOLVERDN_H
#define SA_CUSOLVERDN_H
#include "cublas_v2.h"
typedef struct sa_solver_handle *cusolverDnHandle_t;
typedef int cusolverStatus_t;
cusolverStatus_t cusolverDnCreate(cusolverDnHandle_t *h);
cusolverStatus_t cusolverDnDestroy(cusolverDnHandle_t h);
cusolverStatus_t cusolverDnDpotrf_bufferSize(cusolverDnHandle_t h, cublasFillMode_t u, int n, double *A,
                                             int lda, int *lwork);
cusolverStatus_t cusolverDnDpotrf(cusolverDnHandle_t h, cublasFillMode_t u, int n, double *A, int lda,
                                  double *work, int lwork, int *info);
cusolverStatus_t cusolverDnDpotrs(cusolverDnHandle_t h, cublasFillMode_t u, int n, int nrhs, const double *A,
                                  int lda, double *B, int ldb, int *info);
#endif
