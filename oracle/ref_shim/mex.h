/* MATLAB MEX API stand-in for the CPU build of the reference (TEST INFRASTRUCTURE ONLY). */
#ifndef SA_MEX_H
#define SA_MEX_H
#include <cstddef>
typedef size_t mwSize;
typedef double mxDouble;
typedef struct mxArray_tag {
	size_t m, n;
	void *data;
	int owns;
} mxArray;
enum { mxREAL = 0 };
mxDouble *mxGetDoubles(const mxArray *a);
double mxGetScalar(const mxArray *a);
size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
mxArray *mxCreateDoubleMatrix(size_t m, size_t n, int complexity);
void mxFree(void *p);
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
#endif
