// mp_noalloc.cu -- the allocation-free batch entry point.
//
// Some callers cannot allocate device memory: an application whose GPU
// memory is owned by its own allocator or reserved up front, a plugin hosted
// in such a process, or a latency-critical loop where a cudaMalloc (which can
// synchronise the device) is not acceptable.  For them this file provides
// mpk_pipeline_run_noalloc: the same stages as mpk_pipeline_run, but every
// intermediate image lives in one file-scope device array that is part of
// the library image, and the per-image job descriptors travel as kernel
// parameters, so the call allocates no device memory at all.
//
// The array costs MP_NOALLOC_SCRATCH_BYTES on every GPU that loads the
// library, for the life of the process.  In host code its name is only a
// host-side stand-in: the device address is looked up once per device with
// cudaGetSymbolAddress (with that device current, on the first call on that
// device) and passed to the kernels.  The address is kept for the life of
// the process, so a process that calls cudaDeviceReset (which unloads the
// library's device image) must not use this entry point afterwards.  The
// first call on a device should come before any stream capture.
#include <mutex>
#include <string.h>

#include "mp_internal.cuh"

// Two halves used alternately for the intermediates of one image.
#define MP_NOALLOC_SCRATCH_BYTES (32u << 20)
#define MP_NOALLOC_HALF_BYTES (MP_NOALLOC_SCRATCH_BYTES / 2)
#define MP_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char mp_noalloc_scratch[MP_NOALLOC_SCRATCH_BYTES];
// Error word the kernels of this path report a timed-out wait into.
static __device__ __align__(256) int mp_noalloc_err;

struct MPNoallocDevice {
    bool ready;
    unsigned char *scratch;   // device address of mp_noalloc_scratch
    int *err;                 // device address of mp_noalloc_err
};

static MPNoallocDevice mp_noalloc_dev[MP_NOALLOC_MAX_DEVICES];
static std::mutex mp_noalloc_mutex;

// Once per device, with that device current: resolve the device addresses
// of the file-scope arrays and clear the error word.
static MPStatus mp_noalloc_setup(int dev, MPNoallocDevice *out)
{
    if (dev < 0 || dev >= MP_NOALLOC_MAX_DEVICES) return MP_ERROR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(mp_noalloc_mutex);
    MPNoallocDevice &d = mp_noalloc_dev[dev];
    if (!d.ready) {
        void *scratch = nullptr, *err = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&scratch, mp_noalloc_scratch);
        if (e != cudaSuccess) return mp_cuda_status(e);
        e = cudaGetSymbolAddress(&err, mp_noalloc_err);
        if (e != cudaSuccess) return mp_cuda_status(e);
        const int zero = 0;
        e = cudaMemcpyToSymbol(mp_noalloc_err, &zero, sizeof(int));
        if (e != cudaSuccess) return mp_cuda_status(e);
        d.scratch = (unsigned char *)scratch;
        d.err = (int *)err;
        d.ready = true;
    }
    *out = d;
    return MILLIPYDE_SUCCESS;
}

// Stream-ordered read of this call's error word after its launches, then
// wait for the stream; a set word becomes MP_ERROR_KERNEL_TIMEOUT and is
// cleared.  Runs on every exit path after the first launch, so the call
// never returns with its work still in flight on the caller's buffers.
static MPStatus mp_noalloc_finish(const MPNoallocDevice &d, cudaStream_t s, MPStatus launch_status)
{
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, d.err, sizeof(int), cudaMemcpyDeviceToHost, s);
    const cudaError_t es = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = es;
    if (launch_status != MILLIPYDE_SUCCESS) return launch_status;
    if (e != cudaSuccess) return mp_cuda_status(e);
    if (h != MP_KERR_NONE) {
        e = cudaMemsetAsync(d.err, 0, sizeof(int), s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return mp_cuda_status(e);
        return MP_ERROR_KERNEL_TIMEOUT;
    }
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpk_pipeline_run_noalloc(const MPStage *stages, int nstages, const MPImage *in,
                                             const MPImage *out, int nimgs, uint64_t seed,
                                             uint64_t index0, void *stream)
{
    if (nimgs < 0 || nstages < 0 || (nimgs > 0 && (!in || !out)) || (nstages > 0 && !stages))
        return MP_ERROR_INVALID_ARGS;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return mp_cuda_status(e);
    MPNoallocDevice d;
    MPStatus st = mp_noalloc_setup(dev, &d);
    if (st != MILLIPYDE_SUCCESS) return st;
    cudaStream_t s = (cudaStream_t)stream;
    // 1. validate every image (descriptors, parameters, intermediate sizes)
    //    before anything is launched
    for (int i = 0; i < nimgs; ++i) {
        st = mp_run_image_noalloc(stages, nstages, seed, index0 + (uint64_t)i, in[i], out[i], d.scratch,
                                  d.scratch + MP_NOALLOC_HALF_BYTES, MP_NOALLOC_HALF_BYTES, d.err, s, false);
        if (st != MILLIPYDE_SUCCESS) return st;
    }
    if (nimgs == 0) return MILLIPYDE_SUCCESS;
    // 2. the error word starts at zero for this call: a word left set by an
    //    earlier call (or another caller) is not reported here
    e = cudaMemsetAsync(d.err, 0, sizeof(int), s);
    if (e != cudaSuccess) return mp_cuda_status(e);
    // 3. images one after another, intermediates in the two halves
    for (int i = 0; i < nimgs && st == MILLIPYDE_SUCCESS; ++i)
        st = mp_run_image_noalloc(stages, nstages, seed, index0 + (uint64_t)i, in[i], out[i], d.scratch,
                                  d.scratch + MP_NOALLOC_HALF_BYTES, MP_NOALLOC_HALF_BYTES, d.err, s, true);
    // 4. wait for the work, report a timed-out device-side wait
    return mp_noalloc_finish(d, s, st);
}
