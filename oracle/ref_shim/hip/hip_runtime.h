/*
 * hip_runtime.h -- CPU stand-in for the HIP runtime, used ONLY to compile the
 * reference's own kernel source (src/millipyde_image.cpp) into a host
 * library that produces golden vectors.  Test infrastructure, never product.
 *
 * Kernels run on the CPU: every block of a launch is executed in turn, and
 * the threads of a block are cooperative coroutines (ucontext) so that
 * __syncthreads() is a real barrier.  `__shared__` arrays become function
 * statics, which all coroutines of the running block share.  Device memory
 * is host memory (malloc); copies are memcpy.
 */
#ifndef MP_REF_SHIM_HIP_RUNTIME_H
#define MP_REF_SHIM_HIP_RUNTIME_H

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <functional>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__ static

typedef int hipError_t;
typedef void *hipStream_t;
typedef void *hipDeviceptr_t;
#define hipSuccess 0
enum { hipMemcpyHostToDevice = 1, hipMemcpyDeviceToHost = 2, hipMemcpyDeviceToDevice = 3 };

struct dim3 {
    unsigned x, y, z;
    dim3(double a = 1, double b = 1, double c = 1)
        : x((unsigned)a), y((unsigned)b), z((unsigned)c) {}
};

/* Per-coroutine thread coordinates, set by the scheduler before resuming. */
extern dim3 mpemu_tid, mpemu_bid, mpemu_bdim, mpemu_gdim;
#define hipThreadIdx_x (mpemu_tid.x)
#define hipThreadIdx_y (mpemu_tid.y)
#define hipThreadIdx_z (mpemu_tid.z)
#define hipBlockIdx_x (mpemu_bid.x)
#define hipBlockIdx_y (mpemu_bid.y)
#define hipBlockIdx_z (mpemu_bid.z)
#define hipBlockDim_x (mpemu_bdim.x)
#define hipBlockDim_y (mpemu_bdim.y)
#define hipBlockDim_z (mpemu_bdim.z)

void mpemu_syncthreads();
void mpemu_launch(dim3 grid, dim3 block, std::function<void()> body);
#define __syncthreads() mpemu_syncthreads()

/* The reference calls hipLaunchKernelGGL(kernel, grid, block, smem, stream,
 * args...); template kernels are deduced from the arguments as in HIP. */
#define hipLaunchKernelGGL(kernel, grid, block, smem, stream, ...) \
    mpemu_launch(dim3(grid), dim3(block), [=]() { kernel(__VA_ARGS__); })

static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }

template <class T>
static inline hipError_t hipMalloc(T **p, size_t n)
{
    *p = (T *)malloc(n ? n : 1);
    return *p ? hipSuccess : 2;
}
static inline hipError_t hipFree(void *p) { free(p); return hipSuccess; }
static inline hipError_t hipMemcpy(void *d, const void *s, size_t n, int) { memcpy(d, s, n); return hipSuccess; }
static inline hipError_t hipMemcpyDtoD(void *d, const void *s, size_t n) { memcpy(d, s, n); return hipSuccess; }
static inline hipError_t hipMemcpyToSymbol(const void *sym, const void *s, size_t n)
{
    memcpy((void *)sym, s, n);
    return hipSuccess;
}
#define HIP_SYMBOL(x) ((const void *)&(x))
static inline hipError_t hipSetDevice(int) { return hipSuccess; }
static inline hipError_t hipStreamSynchronize(hipStream_t) { return hipSuccess; }
static inline hipError_t hipDeviceSynchronize() { return hipSuccess; }
static inline const char *hipGetErrorString(hipError_t) { return "emulated"; }

#endif
