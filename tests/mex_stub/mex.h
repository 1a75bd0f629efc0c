/* Test stand-in for MATLAB's MEX API: only the calls the gateways in
 * shape_atrophy_gb300/mex/ make, so the gateways can be compiled and driven
 * without MATLAB (tests/test_gpu_mex_gateway.py). */
#ifndef SA_TEST_MEX_H
#define SA_TEST_MEX_H
#include <cstddef>
typedef size_t mwSize;
typedef double mxDouble;
typedef struct mxArray_tag mxArray;
enum { mxREAL = 0 };
mxDouble *mxGetDoubles(const mxArray *a);
double mxGetScalar(const mxArray *a);
size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
size_t mxGetNumberOfElements(const mxArray *a);
mxArray *mxCreateDoubleMatrix(size_t m, size_t n, int complexity);
void mxFree(void *p);
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
int mexAtExit(void (*f)(void));
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
#endif
