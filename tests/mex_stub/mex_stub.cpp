// Test stand-in for the MEX runtime: mxArrays over caller-owned memory (host, or device memory for the
// gpuArray arguments, as MATLAB passes them), mexErrMsgIdAndTxt as a C++ exception caught by
// stub_call, and a C entry point that runs the gateway's mexFunction.
#include "mex.h"
#include "gpu/mxGPUArray.h"
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

struct mxArray_tag {
	size_t m, n;
	void *data;
	bool owns;
};
struct mxGPUArray_tag {
	const mxArray *a;
};

namespace {
struct MexError : std::runtime_error {
	using std::runtime_error::runtime_error;
};
std::vector<void (*)(void)> g_exit;
}  // namespace

mxDouble *mxGetDoubles(const mxArray *a) { return (mxDouble *) a->data; }
double mxGetScalar(const mxArray *a) { return ((const double *) a->data)[0]; }
size_t mxGetM(const mxArray *a) { return a->m; }
size_t mxGetN(const mxArray *a) { return a->n; }
size_t mxGetNumberOfElements(const mxArray *a) { return a->m * a->n; }
mxArray *mxCreateDoubleMatrix(size_t m, size_t n, int)
{
	mxArray *a = new mxArray{m, n, calloc(m * n ? m * n : 1, sizeof(double)), true};
	return a;
}
void mxFree(void *p) { free(p); }
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...)
{
	char buf[1024];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof buf, fmt, ap);
	va_end(ap);
	throw MexError(std::string(id) + ": " + buf);
}
int mexAtExit(void (*f)(void))
{
	g_exit.push_back(f);
	return 0;
}
int mxInitGPU(void) { return 0; }
const mxGPUArray *mxGPUCreateFromMxArray(const mxArray *a) { return new mxGPUArray{a}; }
const void *mxGPUGetDataReadOnly(const mxGPUArray *g) { return g->a->data; }
const mwSize *mxGPUGetDimensions(const mxGPUArray *g)
{
	mwSize *d = (mwSize *) malloc(2 * sizeof(mwSize));
	d[0] = g->a->m;
	d[1] = g->a->n;
	return d;
}
void mxGPUDestroyGPUArray(const mxGPUArray *g) { delete g; }

extern "C" {
mxArray *stub_wrap(size_t m, size_t n, void *data) { return new mxArray{m, n, data, false}; }
void *stub_data(mxArray *a) { return a->data; }
void stub_free(mxArray *a)
{
	if (a && a->owns) free(a->data);
	delete a;
}
int stub_call(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs, char *err, int errLen)
{
	try {
		mexFunction(nlhs, plhs, nrhs, prhs);
		return 0;
	} catch (const std::exception &e) {
		if (err && errLen > 0) snprintf(err, (size_t) errLen, "%s", e.what());
		return 1;
	}
}
void stub_atexit(void)
{
	for (auto f : g_exit) f();
	g_exit.clear();
}
}
