/* Test stand-in for MATLAB's mxGPUArray API (see ../mex.h). */
#ifndef SA_TEST_MXGPUARRAY_H
#define SA_TEST_MXGPUARRAY_H
#include "../mex.h"
typedef struct mxGPUArray_tag mxGPUArray;
int mxInitGPU(void);
const mxGPUArray *mxGPUCreateFromMxArray(const mxArray *a);
const void *mxGPUGetDataReadOnly(const mxGPUArray *a);
const mwSize *mxGPUGetDimensions(const mxGPUArray *a);
void mxGPUDestroyGPUArray(const mxGPUArray *a);
#endif
