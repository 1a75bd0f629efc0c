/*
 * cuda_emu.h -- force-included when the reference's CUDA sources are
 * compiled for the CPU (oracle/build_ref.py).  TEST INFRASTRUCTURE ONLY.
 *
 * Kernels run as plain loops over (block, thread); kernels that call
 * __syncthreads run each thread of a block as a fiber so the barrier has
 * CUDA semantics.  __shared__ locals become function statics (one copy
 * shared by the threads of the block being run).
 */
#ifndef SA_CUDA_EMU_H
#define SA_CUDA_EMU_H
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <cstdio>
#include <cfloat>
#include <functional>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__ static

struct double2 { double x, y; };
struct double3 { double x, y, z; };
struct uint3 { unsigned int x, y, z; };
struct dim3 {
	unsigned int x, y, z;
	dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};

extern thread_local uint3 threadIdx, blockIdx;
extern thread_local dim3 blockDim, gridDim;

void sa_emu_launch(dim3 g, dim3 b, const std::function<void()> &body, bool needs_barrier);
void __syncthreads();

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2,
                      cudaMemcpyDeviceToDevice = 3, cudaMemcpyDefault = 4 };
typedef int cudaEvent_t;

cudaError_t cudaMalloc(void **p, size_t n);
cudaError_t cudaFree(void *p);
cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind k);
cudaError_t cudaMemset(void *d, int v, size_t n);
cudaError_t cudaEventCreate(cudaEvent_t *e);
cudaError_t cudaEventRecord(cudaEvent_t e);
cudaError_t cudaEventSynchronize(cudaEvent_t e);
cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t a, cudaEvent_t b);
cudaError_t cudaEventDestroy(cudaEvent_t e);

template <class T>
cudaError_t cudaMemcpyToSymbol(T &sym, const void *src, size_t n, size_t off = 0,
                               cudaMemcpyKind k = cudaMemcpyHostToDevice)
{ (void) k; memcpy((char *) &sym + off, src, n); return cudaSuccess; }

template <class T>
cudaError_t cudaMemcpyFromSymbol(void *dst, const T &sym, size_t n, size_t off = 0,
                                 cudaMemcpyKind k = cudaMemcpyDeviceToHost)
{ (void) k; memcpy(dst, (const char *) &sym + off, n); return cudaSuccess; }

#endif
