/* mxGPUArray stand-in for the CPU build of the reference (TEST INFRASTRUCTURE ONLY). */
#ifndef SA_MXGPUARRAY_H
#define SA_MXGPUARRAY_H
#include "../mex.h"
typedef mxArray mxGPUArray;
int mxInitGPU(void);
const mxGPUArray *mxGPUCreateFromMxArray(const mxArray *a);
const void *mxGPUGetDataReadOnly(const mxGPUArray *a);
const mwSize *mxGPUGetDimensions(const mxGPUArray *a);
void mxGPUDestroyGPUArray(const mxGPUArray *a);
#endif
