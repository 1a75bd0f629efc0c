/*
 * emu_runtime.cpp -- CPU runtime for the reference's CUDA sources
 * (TEST INFRASTRUCTURE ONLY; see oracle/build_ref.py).
 *
 * Provides: kernel launch emulation (plain loops; fibers for kernels with
 * __syncthreads), the CUDA runtime calls the reference makes, textbook
 * cuBLAS / cuSOLVER routines whose summation order matches the oracle's
 * dense routines, and the MATLAB MEX API pieces the gateways use.  The
 * entry point sa_ref_mex() calls the reference's own mexFunction.
 */
#include "cuda_emu.h"
#include "cublas_v2.h"
#include "cusolverDn.h"
#include "mex.h"
#include "gpu/mxGPUArray.h"
#include <ucontext.h>
#include <cstdarg>
#include <csetjmp>
#include <vector>

thread_local uint3 threadIdx, blockIdx;
thread_local dim3 blockDim, gridDim;

/* ---------------- kernel launch ---------------- */
namespace {
struct Fiber {
	ucontext_t ctx;
	std::vector<char> stack;
	bool done;
	uint3 tid;
};
ucontext_t g_sched;
Fiber *g_cur = nullptr;
const std::function<void()> *g_body = nullptr;

void fiber_entry()
{
	threadIdx = g_cur->tid;
	(*g_body)();
	g_cur->done = true;
	swapcontext(&g_cur->ctx, &g_sched);
}
}   // namespace

void __syncthreads()
{
	if (g_cur) swapcontext(&g_cur->ctx, &g_sched);
}

void sa_emu_launch(dim3 g, dim3 b, const std::function<void()> &body, bool needs_barrier)
{
	gridDim = g;
	blockDim = b;
	for (unsigned bz = 0; bz < g.z; ++bz)
	for (unsigned by = 0; by < g.y; ++by)
	for (unsigned bx = 0; bx < g.x; ++bx) {
		blockIdx = {bx, by, bz};
		if (!needs_barrier) {
			for (unsigned tz = 0; tz < b.z; ++tz)
			for (unsigned ty = 0; ty < b.y; ++ty)
			for (unsigned tx = 0; tx < b.x; ++tx) {
				threadIdx = {tx, ty, tz};
				body();
			}
			continue;
		}
		size_t nt = (size_t) b.x * b.y * b.z;
		std::vector<Fiber> fib(nt);
		size_t k = 0;
		for (unsigned tz = 0; tz < b.z; ++tz)
		for (unsigned ty = 0; ty < b.y; ++ty)
		for (unsigned tx = 0; tx < b.x; ++tx, ++k) {
			Fiber &f = fib[k];
			f.stack.resize(64 * 1024);
			f.done = false;
			f.tid = {tx, ty, tz};
			getcontext(&f.ctx);
			f.ctx.uc_stack.ss_sp = f.stack.data();
			f.ctx.uc_stack.ss_size = f.stack.size();
			f.ctx.uc_link = &g_sched;
			makecontext(&f.ctx, fiber_entry, 0);
		}
		g_body = &body;
		bool left = true;
		while (left) {      /* run every thread up to its next barrier, in thread order */
			left = false;
			for (auto &f : fib) {
				if (f.done) continue;
				g_cur = &f;
				threadIdx = f.tid;
				swapcontext(&g_sched, &f.ctx);
				g_cur = nullptr;
				if (!f.done) left = true;
			}
		}
	}
}

/* ---------------- runtime ---------------- */
cudaError_t cudaMalloc(void **p, size_t n)
{
	*p = calloc(n ? n : 1, 1);
	return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void *p) { free(p); return cudaSuccess; }
cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { memmove(d, s, n); return cudaSuccess; }
cudaError_t cudaMemset(void *d, int v, size_t n) { memset(d, v, n); return cudaSuccess; }
cudaError_t cudaEventCreate(cudaEvent_t *e) { *e = 0; return cudaSuccess; }
cudaError_t cudaEventRecord(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t, cudaEvent_t) { *ms = 0.0f; return cudaSuccess; }
cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }

/* ---------------- cuBLAS (textbook order) ---------------- */
cublasStatus_t cublasCreate(cublasHandle_t *h) { *h = nullptr; return 0; }
cublasStatus_t cublasDestroy(cublasHandle_t) { return 0; }

cublasStatus_t cublasDdot(cublasHandle_t, int n, const double *x, int incx, const double *y, int incy,
                          double *result)
{
	double s = 0.0;
	for (int i = 0; i < n; ++i) s += x[(size_t) i * incx] * y[(size_t) i * incy];
	*result = s;
	return 0;
}

cublasStatus_t cublasDgemv(cublasHandle_t, cublasOperation_t t, int m, int n, const double *alpha,
                           const double *A, int lda, const double *x, int incx, const double *beta,
                           double *y, int incy)
{
	if (t != CUBLAS_OP_N) return 1;
	for (int i = 0; i < m; ++i) {
		double s = 0.0;
		for (int j = 0; j < n; ++j) s += A[(size_t) j * lda + i] * x[(size_t) j * incx];
		double &yi = y[(size_t) i * incy];
		yi = (*beta == 0.0 ? *alpha * s : *alpha * s + *beta * yi);
	}
	return 0;
}

cublasStatus_t cublasDgemm(cublasHandle_t, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                           const double *alpha, const double *A, int lda, const double *B, int ldb,
                           const double *beta, double *C, int ldc)
{
	if (ta != CUBLAS_OP_N || tb != CUBLAS_OP_N) return 1;
	for (int c = 0; c < n; ++c)
		for (int i = 0; i < m; ++i) {
			double s = 0.0;
			for (int p = 0; p < k; ++p) s += A[(size_t) p * lda + i] * B[(size_t) c * ldb + p];
			double &ci = C[(size_t) c * ldc + i];
			ci = (*beta == 0.0 ? *alpha * s : *alpha * s + *beta * ci);
		}
	return 0;
}

/* ---------------- cuSOLVER (textbook Cholesky) ---------------- */
cusolverStatus_t cusolverDnCreate(cusolverDnHandle_t *h) { *h = nullptr; return 0; }
cusolverStatus_t cusolverDnDestroy(cusolverDnHandle_t) { return 0; }
cusolverStatus_t cusolverDnDpotrf_bufferSize(cusolverDnHandle_t, cublasFillMode_t, int, double *, int, int *lw)
{ *lw = 1; return 0; }

cusolverStatus_t cusolverDnDpotrf(cusolverDnHandle_t, cublasFillMode_t u, int n, double *A, int lda,
                                  double *, int, int *info)
{
	if (u != CUBLAS_FILL_MODE_LOWER) return 1;
	std::vector<double> L((size_t) n * n);
	int bad = 0;
	for (int j = 0; j < n; ++j) {
		double s = A[(size_t) j * lda + j];
		const double *Lj = &L[(size_t) j * n];
		for (int k = 0; k < j; ++k) s -= Lj[k] * Lj[k];
		if (!(s > 0.0) && !bad) bad = j + 1;
		double ljj = std::sqrt(s);
		L[(size_t) j * n + j] = ljj;
		for (int i = j + 1; i < n; ++i) {
			const double *Li = &L[(size_t) i * n];
			double t = A[(size_t) j * lda + i];
			for (int k = 0; k < j; ++k) t -= Li[k] * Lj[k];
			L[(size_t) i * n + j] = t / ljj;
		}
	}
	for (int j = 0; j < n; ++j)
		for (int i = j; i < n; ++i) A[(size_t) j * lda + i] = L[(size_t) i * n + j];
	*info = bad;
	return 0;
}

cusolverStatus_t cusolverDnDpotrs(cusolverDnHandle_t, cublasFillMode_t u, int n, int nrhs, const double *A,
                                  int lda, double *B, int ldb, int *info)
{
	if (u != CUBLAS_FILL_MODE_LOWER) return 1;
	for (int c = 0; c < nrhs; ++c) {
		double *b = B + (size_t) c * ldb;
		for (int i = 0; i < n; ++i) {
			double s = b[i];
			for (int k = 0; k < i; ++k) s -= A[(size_t) k * lda + i] * b[k];
			b[i] = s / A[(size_t) i * lda + i];
		}
		for (int i = n - 1; i >= 0; --i) {
			double s = b[i];
			const double *Li = A + (size_t) i * lda;
			for (int k = i + 1; k < n; ++k) s -= Li[k] * b[k];
			b[i] = s / Li[i];
		}
	}
	*info = 0;
	return 0;
}

/* ---------------- MEX ---------------- */
static jmp_buf g_mexjmp;
static char g_mexmsg[512];

mxDouble *mxGetDoubles(const mxArray *a) { return (mxDouble *) a->data; }
double mxGetScalar(const mxArray *a) { return ((const double *) a->data)[0]; }
size_t mxGetM(const mxArray *a) { return a->m; }
size_t mxGetN(const mxArray *a) { return a->n; }
mxArray *mxCreateDoubleMatrix(size_t m, size_t n, int)
{
	mxArray *a = (mxArray *) calloc(1, sizeof(mxArray));
	a->m = m; a->n = n;
	a->data = calloc(m * n ? m * n : 1, sizeof(double));
	a->owns = 1;
	return a;
}
void mxFree(void *p) { free(p); }
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	int k = snprintf(g_mexmsg, sizeof(g_mexmsg), "%s: ", id);
	vsnprintf(g_mexmsg + k, sizeof(g_mexmsg) - k, fmt, ap);
	va_end(ap);
	longjmp(g_mexjmp, 1);
}
int mxInitGPU(void) { return 0; }
const mxGPUArray *mxGPUCreateFromMxArray(const mxArray *a) { return a; }
const void *mxGPUGetDataReadOnly(const mxGPUArray *a) { return a->data; }
const mwSize *mxGPUGetDimensions(const mxGPUArray *a)
{
	mwSize *d = (mwSize *) malloc(2 * sizeof(mwSize));
	d[0] = a->m; d[1] = a->n;
	return d;
}
void mxGPUDestroyGPUArray(const mxGPUArray *) {}

/* ---------------- entry points for ctypes ---------------- */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, mxArray const *prhs[]);

extern "C" {
/* wrap caller memory (no copy); MATLAB matrix m x n, column-major */
mxArray *sa_ref_wrap(size_t m, size_t n, void *data)
{
	mxArray *a = (mxArray *) calloc(1, sizeof(mxArray));
	a->m = m; a->n = n; a->data = data; a->owns = 0;
	return a;
}
void *sa_ref_data(mxArray *a) { return a->data; }
void sa_ref_free(mxArray *a)
{
	if (!a) return;
	if (a->owns) free(a->data);
	free(a);
}
const char *sa_ref_error(void) { return g_mexmsg; }
/* returns 0 on success, 1 when the gateway raised a MEX error */
int sa_ref_mex(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs)
{
	g_mexmsg[0] = 0;
	if (setjmp(g_mexjmp)) return 1;
	mexFunction(nlhs, plhs, nrhs, prhs);
	return 0;
}
}
