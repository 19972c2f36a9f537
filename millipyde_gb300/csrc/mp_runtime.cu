// mp_runtime.cu -- device layer, object memory, status strings and RNG.
//
// Replaces, for one GPU per process:
//   src/millipyde_devices.cpp   device discovery, per-device streams
//   src/millipyde_objects.cpp   alloc / H2D / D2H / clone of MPObjData
//   src/millipyde.c             mperr_str, random_*_in_range
// Differences that matter to callers: nothing here exits the process; device
// memory comes from the device's stream-ordered pool (cudaMallocAsync) with a
// retained release threshold, so per-op allocations are cheap; each device
// has one non-blocking library stream that objects are ordered on.
#include <algorithm>
#include <atomic>
#include <deque>
#include <mutex>
#include <vector>
#include <string.h>
#include <stdio.h>
#include <stdlib.h>
#include <time.h>
#include <limits.h>

#include "mp_internal.cuh"

#define MP_MAX_DEVICES 64

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------
static thread_local char mp_err_text[256];

void mp_set_cuda_error(cudaError_t e)
{
    snprintf(mp_err_text, sizeof(mp_err_text), "%s: %s", cudaGetErrorName(e),
             cudaGetErrorString(e));
}

MPStatus mp_cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return MILLIPYDE_SUCCESS;
    mp_set_cuda_error(e);
    cudaGetLastError();   // clear a non-sticky error so the next call does not report it
    if (e == cudaErrorMemoryAllocation) return MP_ERROR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return MP_ERROR_NO_DEVICE;
    return MP_ERROR_CUDA;
}

extern "C" const char *mp_last_cuda_error(void) { return mp_err_text; }

extern "C" const char *mperr_str(MPStatus status)
{
    switch (status) {
    case MILLIPYDE_SUCCESS: return "success";
    case MOD_ERROR: return "module 'millipyde' could not be created";
    case MOD_ERROR_CREATE_GPUARRAY_TYPE: return "could not ready type 'gpuarray'";
    case MOD_ERROR_CREATE_GPUIMAGE_TYPE: return "could not ready type 'gpuimage'";
    case MOD_ERROR_CREATE_OPERATION_TYPE: return "could not ready type 'Operation'";
    case MOD_ERROR_CREATE_PIPELINE_TYPE: return "could not ready type 'Pipeline'";
    case MOD_ERROR_CREATE_DEVICE_TYPE: return "could not ready type 'Device'";
    case MOD_ERROR_CREATE_GENERATOR_TYPE: return "could not ready type 'Generator'";
    case MOD_ERROR_ADD_GPUARRAY: return "could not add type 'gpuarray' to the module";
    case MOD_ERROR_ADD_GPUIMAGE: return "could not add type 'gpuimage' to the module";
    case MOD_ERROR_ADD_OPERATION: return "could not add type 'Operation' to the module";
    case MOD_ERROR_ADD_PIPELINE: return "could not add type 'Pipeline' to the module";
    case MOD_ERROR_ADD_DEVICE: return "could not add type 'Device' to the module";
    case MOD_ERROR_ADD_GENERATOR: return "could not add type 'Generator' to the module";
    case DEV_ERROR_CURRENT_DEVICE: return "the CUDA runtime could not report the current device";
    case DEV_ERROR_DEVICE_COUNT: return "the CUDA runtime could not count devices";
    case DEV_ERROR_DEVICE_PROPERTIES: return "the CUDA runtime could not read device properties";
    case DEV_ERROR_PEER_ACCESS_MATRIX_ALLOC: return "could not allocate the peer-access table";
    case DEV_ERROR_DEVICE_ARRAY_ALLOC: return "could not allocate the device table";
    case DEV_WARN_NO_PEER_ACCESS: return "devices cannot access each other's memory";
    case DEV_WARN_BAD_DEVICE: return "device id is not usable";
    case WORK_ERROR_INIT_PTHREAD:
    case WORK_ERROR_INIT_COND:
    case WORK_ERROR_INIT_MUX:
    case WORK_ERROR_ALLOC_WORK_POOL:
    case WORK_ERROR_ALLOC_WORK_NODE:
    case WORK_ERROR_NULL_WORK_POOL: return "work pool error (no work pool in this library)";
    case TYPE_ERROR_NON_GPUOBJ: return "GPU operations need a gpuarray or gpuimage";
    case RAND_ERROR_INSUFFICIENT_BYTES: return "random number generation failed";
    case GPUARRAY_ERROR_CONSTRUCTION_WITHOUT_ARRAY_TYPE:
        return "gpuarray needs an ndarray or an array-like argument";
    case GPUARRAY_ERROR_CONSTRUCTION_WITHOUT_NUMERIC_ARRAY:
        return "gpuarray needs a numeric array";
    case GPUIMAGE_ERROR_CONSTRUCTION_WITHOUT_ARRAY_TYPE:
        return "gpuimage needs an ndarray or an array-like argument";
    case GPUIMAGE_ERROR_CONSTRUCTION_WITHOUT_IMAGE_FORMAT:
        return "gpuimage needs a numeric image array";
    case GPUIMAGE_ERROR_CONSTRUCTION_WITHOUT_IMAGE_DIMS:
        return "gpuimage needs a 2-D array (greyscale) or a 3-D array (height, width, channels)";
    case GPUOPERATION_ERROR_CONSTRUCTION_NO_ARGS:
        return "Operation needs a method name or a callable as its first argument";
    case GPUOPERATION_ERROR_INVALID_PROBABILITY:
        return "Operation probability must be a float strictly between 0 and 1";
    case GPUOPERATION_ERROR_CONSTRUCTION_NAMED_ARGS:
        return "Operation accepts one keyword argument, 'probability'";
    case GPUOPERATION_ERROR_RUN_WITHOUT_STRING_METHOD:
        return "run_on needs an Operation built from a method name";
    case GPUOPERATION_ERROR_RUN_UNKNOWN_STRING_METHOD:
        return "the Operation's method name is not a method of the given object";
    case GPUOPERATION_ERROR_RUN_NO_DEV_RANDOM:
    case GPUOPERATION_ERROR_RUN_CANNOT_READ_DEV_RANDOM: return "random source unavailable";
    case GPUPIPELINE_ERROR_CONSTRUCTION_INVALID_ARGS:
        return "Pipeline takes (inputs, operations) and an optional device";
    case GPUPIPELINE_ERROR_INVALID_DEVICE: return "Pipeline device must be an integer";
    case GPUPIPELINE_ERROR_UNUSABLE_DEVICE: return "Pipeline device is not a usable GPU";
    case GPUPIPELINE_ERROR_CONSTRUCTION_NAMED_ARGS:
        return "Pipeline accepts one keyword argument, 'device'";
    case GPUPIPELINE_ERROR_NONLIST_INPUTS: return "Pipeline inputs must be a list";
    case GPUPIPELINE_ERROR_NONLIST_OPERATIONS: return "Pipeline operations must be a list";
    case GPUPIPELINE_ERROR_NONGPU_INPUT: return "Pipeline inputs must be gpuimages";
    case GPUGENERATOR_ERROR_INVALID_DEVICE: return "Generator device must be an integer";
    case GPUGENERATOR_ERROR_INVALID_MAX:
        return "Generator outputs must be a non-negative integer";
    case GPUGENERATOR_ERROR_INVALID_RETURN_TO: return "Generator return_to_host must be a bool";
    case GPUGENERATOR_ERROR_UNUSABLE_DEVICE: return "Generator device is not a usable GPU";
    case GPUGENERATOR_ERROR_CONSTRUCTION_NAMED_ARGS:
        return "Generator accepts the keyword arguments device, outputs, return_to_host and seed";
    case GPUGENERATOR_ERROR_INVALID_INPUT:
        return "Generator inputs must be a list of images or a directory path";
    case GPUGENERATOR_ERROR_NONLIST_OPERATIONS: return "Generator operations must be a list";
    case MP_ERROR_NO_DEVICE: return "no CUDA device is available";
    case MP_ERROR_CUDA: return "a CUDA runtime call failed";
    case MP_ERROR_OUT_OF_MEMORY: return "out of device memory";
    case MP_ERROR_INVALID_ARGS: return "invalid argument value";
    case MP_ERROR_UNSUPPORTED_TYPE: return "unsupported image dtype or channel count for this operation";
    case MP_ERROR_UNSUPPORTED_DIMS: return "unsupported image dimensions";
    case MP_ERROR_NULL_DATA: return "object has no device data";
    case MP_ERROR_KERNEL_TIMEOUT: return "a device-side wait timed out";
    case MP_ERROR_BAD_DESCRIPTOR: return "malformed batch descriptor";
    case MP_ERROR_TOO_LARGE: return "request exceeds a documented size limit";
    default: return "unknown failure";
    }
}

// ---------------------------------------------------------------------------
// Devices and streams
// ---------------------------------------------------------------------------
static std::mutex mp_dev_mutex;
static int mp_dev_count = -1;
static int mp_target_device = DEVICE_LOC_NO_AFFINITY;
static cudaStream_t mp_streams[MP_MAX_DEVICES];
static int *mp_err_words[MP_MAX_DEVICES];

extern "C" MPStatus mpdev_initialize(void)
{
    std::lock_guard<std::mutex> lk(mp_dev_mutex);
    if (mp_dev_count >= 0) return mp_dev_count > 0 ? MILLIPYDE_SUCCESS : MP_ERROR_NO_DEVICE;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n <= 0) {
        cudaGetLastError();
        mp_dev_count = 0;
        return MP_ERROR_NO_DEVICE;
    }
    if (n > MP_MAX_DEVICES) n = MP_MAX_DEVICES;
    mp_dev_count = n;
    return MILLIPYDE_SUCCESS;
}

extern "C" int mpdev_get_device_count(void)
{
    mpdev_initialize();
    return mp_dev_count;
}

extern "C" int mpdev_get_recommended_device(void) { return mpdev_get_device_count() > 0 ? 0 : HOST_LOC; }

extern "C" int mpdev_get_target_device(void) { return mp_target_device; }

extern "C" void mpdev_set_target_device(int device_id) { mp_target_device = device_id; }

extern "C" MPBool mpdev_is_valid_device(int device_id)
{
    return (device_id >= 0 && device_id < mpdev_get_device_count()) ? MP_TRUE : MP_FALSE;
}

// Lazily creates the device's library stream, its error word, and sets the
// device's memory pool to retain freed memory.
static MPStatus mp_device_setup(int d)
{
    if (!mpdev_is_valid_device(d)) return MP_ERROR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(mp_dev_mutex);
    if (mp_streams[d]) return MILLIPYDE_SUCCESS;
    int prev = 0;
    cudaGetDevice(&prev);
    MP_CUDA_TRY(cudaSetDevice(d));
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, d) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    int *w = nullptr;
    cudaError_t e = cudaMalloc(&w, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(w, 0, 4 * sizeof(int));
    cudaStream_t s = nullptr;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return mp_cuda_status(e);
    mp_err_words[d] = w;
    mp_streams[d] = s;
    return MILLIPYDE_SUCCESS;
}

extern "C" void *mpdev_get_stream(int device_id, int stream_id)
{
    (void)stream_id;
    if (mp_device_setup(device_id) != MILLIPYDE_SUCCESS) return nullptr;
    return (void *)mp_streams[device_id];
}

int *mp_device_error_word(int device)
{
    if (mp_device_setup(device) != MILLIPYDE_SUCCESS) return nullptr;
    return mp_err_words[device];
}

MPStatus mp_check_device_error(cudaStream_t stream)
{
    int d = 0;
    cudaGetDevice(&d);
    int *w = mp_device_error_word(d);
    if (!w) return MP_ERROR_NO_DEVICE;
    int h = 0;
    MP_CUDA_TRY(cudaMemcpyAsync(&h, w, sizeof(int), cudaMemcpyDeviceToHost, stream));
    MP_CUDA_TRY(cudaStreamSynchronize(stream));
    if (h != MP_KERR_NONE) {
        cudaMemsetAsync(w, 0, sizeof(int), stream);
        return MP_ERROR_KERNEL_TIMEOUT;
    }
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpdev_get_device_name(int device_id, char *buf, int len)
{
    if (!buf || len <= 0) return MP_ERROR_INVALID_ARGS;
    buf[0] = 0;
    if (!mpdev_is_valid_device(device_id)) return MP_ERROR_NO_DEVICE;
    cudaDeviceProp prop;
    MP_CUDA_TRY(cudaGetDeviceProperties(&prop, device_id));
    snprintf(buf, (size_t)len, "%s", prop.name);
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpdev_synchronize(void)
{
    int n = mpdev_get_device_count();
    if (n <= 0) return MP_ERROR_NO_DEVICE;
    for (int d = 0; d < n; ++d) {
        if (!mp_streams[d]) continue;
        MP_CUDA_TRY(cudaSetDevice(d));
        MPStatus st = mp_check_device_error(mp_streams[d]);
        if (st != MILLIPYDE_SUCCESS) return st;
    }
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpdev_stream_synchronize(void *stream)
{
    MP_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    return MILLIPYDE_SUCCESS;
}

// Largest single device allocation the library makes (0: no limit); set by
// mpdev_set_alloc_limit to exercise the out-of-memory paths on the host.
static std::atomic<size_t> mp_alloc_limit{0};

extern "C" void mpdev_set_alloc_limit(size_t max_request_bytes) { mp_alloc_limit.store(max_request_bytes); }

MPStatus mp_malloc_async(void **p, size_t bytes, cudaStream_t s)
{
    *p = nullptr;
    if (bytes == 0) return MILLIPYDE_SUCCESS;
    const size_t lim = mp_alloc_limit.load();
    if (lim && bytes > lim) return MP_ERROR_OUT_OF_MEMORY;
    return mp_cuda_status(cudaMallocAsync(p, bytes, s));
}

// ---------------------------------------------------------------------------
// Host-to-device uploads of plan tables through a page-locked ring.  A copy
// from pageable memory may wait for the stream's earlier work before it
// starts (the driver stages it through its own page-locked buffer), which
// would serialise the host's planning of the next batch with the device's
// execution of the last.  The ring is one page-locked block per device,
// handed out in order; a slot is reused only after the event recorded
// behind its copy has completed, which by then it normally has (a whole lap
// of uploads later).  Uploads while the stream is being captured, and
// uploads larger than a quarter of the ring, copy directly: a captured copy
// from the ring would replay whatever the slot holds later.
// ---------------------------------------------------------------------------
#define MP_RING_BYTES ((size_t)32 << 20)

struct MPRingSlot {
    size_t off, bytes;
    unsigned long long lap;
    cudaEvent_t ev;
};

struct MPRing {
    unsigned char *base = nullptr;
    bool failed = false;
    size_t head = 0;
    unsigned long long lap = 0;
    std::deque<MPRingSlot> busy;      // oldest first
    std::vector<cudaEvent_t> spare;
};

static std::mutex mp_ring_mutex;
static MPRing mp_rings[MP_MAX_DEVICES];

static MPStatus mp_ring_retire(MPRing &R, const MPRingSlot &sl)
{
    MP_CUDA_TRY(cudaEventSynchronize(sl.ev));
    R.spare.push_back(sl.ev);
    return MILLIPYDE_SUCCESS;
}

MPStatus mp_upload_async(void *dst, const void *src, size_t bytes, cudaStream_t s)
{
    if (bytes == 0) return MILLIPYDE_SUCCESS;
    int d = 0;
    cudaGetDevice(&d);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
        cudaGetLastError();
        cs = cudaStreamCaptureStatusActive;
    }
    const size_t need = (bytes + 255) & ~(size_t)255;
    if (cs != cudaStreamCaptureStatusNone || d < 0 || d >= MP_MAX_DEVICES || need > MP_RING_BYTES / 4)
        return mp_cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
    std::lock_guard<std::mutex> lk(mp_ring_mutex);
    MPRing &R = mp_rings[d];
    if (!R.base && !R.failed) {
        if (cudaHostAlloc((void **)&R.base, MP_RING_BYTES, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            R.base = nullptr;
            R.failed = true;
        }
    }
    if (!R.base) return mp_cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
    if (R.head + need > MP_RING_BYTES) {
        // wrap: the previous lap's slots past this lap's end are retired
        // now, so that only this lap's slots (in offset order) stay queued
        while (!R.busy.empty() && R.busy.front().lap < R.lap) {
            MPStatus st = mp_ring_retire(R, R.busy.front());
            R.busy.pop_front();
            if (st != MILLIPYDE_SUCCESS) return st;
        }
        R.head = 0;
        ++R.lap;
    }
    const size_t lo = R.head, hi = R.head + need;
    while (!R.busy.empty() && R.busy.front().lap < R.lap && R.busy.front().off < hi) {
        MPStatus st = mp_ring_retire(R, R.busy.front());
        R.busy.pop_front();
        if (st != MILLIPYDE_SUCCESS) return st;
    }
    cudaEvent_t ev = nullptr;
    if (!R.spare.empty()) {
        ev = R.spare.back();
        R.spare.pop_back();
    } else {
        MP_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    }
    memcpy(R.base + lo, src, bytes);
    cudaError_t e = cudaMemcpyAsync(dst, R.base + lo, bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        R.spare.push_back(ev);
        return mp_cuda_status(e);
    }
    e = cudaEventRecord(ev, s);
    if (e != cudaSuccess) {
        // the copy is queued but nothing marks its end: wait for it before
        // the slot can be handed out again
        R.spare.push_back(ev);
        cudaStreamSynchronize(s);
        return mp_cuda_status(e);
    }
    R.busy.push_back(MPRingSlot{lo, need, R.lap, ev});
    R.head = hi;
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpdev_pool_usage(int device_id, uint64_t *reserved, uint64_t *used, uint64_t *used_peak)
{
    if (!reserved || !used) return MP_ERROR_INVALID_ARGS;
    if (!mpdev_is_valid_device(device_id)) return MP_ERROR_NO_DEVICE;
    cudaMemPool_t pool;
    MP_CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, device_id));
    cuuint64_t r = 0, u = 0, h = 0;
    MP_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &r));
    MP_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &u));
    MP_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &h));
    *reserved = (uint64_t)r;
    *used = (uint64_t)u;
    if (used_peak) *used_peak = (uint64_t)h;
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpdev_pool_reset_peak(int device_id)
{
    if (!mpdev_is_valid_device(device_id)) return MP_ERROR_NO_DEVICE;
    cudaMemPool_t pool;
    MP_CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, device_id));
    cuuint64_t zero = 0;
    MP_CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero));
    return MILLIPYDE_SUCCESS;
}

// ---------------------------------------------------------------------------
// Self-test of the bounded device-side wait: one CTA waits on an mbarrier
// phase that never completes (two arrivals expected, one made; no copy is
// involved), gives up after `polls` polls through the same wait the kernels
// use, and reports MP_KERR_TIMEOUT into the device's error word.
// ---------------------------------------------------------------------------
__global__ void mp_selftest_wait_kernel(int *err, uint32_t polls)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mp_mbar_init(&bar, 2);
        mp_fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(mp_smem_addr(&bar)) : "memory");
    }
    const bool ok = mp_mbar_wait_bounded(&bar, 0, polls);
    if (!__syncthreads_and(ok) && threadIdx.x == 0) atomicExch(err, MP_KERR_TIMEOUT);
}

extern "C" MPStatus mpdev_selftest_wait_timeout(uint32_t polls, void *stream)
{
    int d = 0;
    MP_CUDA_TRY(cudaGetDevice(&d));
    int *w = mp_device_error_word(d);
    if (!w) return MP_ERROR_NO_DEVICE;
    if (polls == 0 || polls > MP_SPIN_LIMIT) return MP_ERROR_INVALID_ARGS;
    cudaStream_t s = (cudaStream_t)stream;
    mp_selftest_wait_kernel<<<1, 32, 0, s>>>(w, polls);
    MP_CUDA_TRY(cudaGetLastError());
    return mp_check_device_error(s);
}

void mp_free_async(void *p, cudaStream_t s)
{
    if (p) cudaFreeAsync(p, s);
}

// ---------------------------------------------------------------------------
// Tensor-map encoder, looked up from the driver at run time (no -lcuda).
// ---------------------------------------------------------------------------
mp_encode_tiled_fn mp_get_encode_tiled()
{
    static mp_encode_tiled_fn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, []() {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (mp_encode_tiled_fn)p;
        else
            cudaGetLastError();
    });
    return fn;
}

// ---------------------------------------------------------------------------
// Object memory
// ---------------------------------------------------------------------------
extern "C" int mp_type_itemsize(int type)
{
    switch (type) {
    case 0: case 1: case 2: return 1;          // bool, int8, uint8
    case 3: case 4: case 23: return 2;         // int16, uint16, float16
    case 5: case 6: case 11: return 4;         // int32, uint32, float32
    case 7: case 8: case 9: case 10: case 12: case 14: return 8;
    case 13: case 15: return 16;
    case 16: return 32;
    default: return 0;
    }
}

static size_t mp_row_bytes(const MPObjData *o, int itemsize)
{
    size_t rb = (size_t)itemsize;
    for (int i = 1; i < o->ndims; ++i) rb *= (size_t)o->dims[i];
    return rb;
}

static int mp_obj_itemsize(const MPObjData *o)
{
    // The innermost stride is the item size for every layout this library makes.
    if (o->ndims >= 1) return o->dims[2 * o->ndims - 1];
    return mp_type_itemsize(o->type);
}

extern "C" size_t mpobj_host_nbytes(const MPObjData *o)
{
    if (!o) return 0;
    size_t n = (size_t)mp_obj_itemsize(o);
    for (int i = 0; i < o->ndims; ++i) n *= (size_t)o->dims[i];
    return n;
}

static int mp_pick_device(void)
{
    int d = mpdev_get_target_device();
    if (d == DEVICE_LOC_NO_AFFINITY || !mpdev_is_valid_device(d)) d = mpdev_get_recommended_device();
    return d;
}

// ---------------------------------------------------------------------------
// Host <-> device copies of object data: `rows` rows of `rowbytes` bytes
// between a packed host buffer and device rows `pitch` bytes apart, on
// stream s, returning after the copy.  Measured on GB300 (a 108 MB image of
// pitched rows, pageable numpy memory): host -> device straight from
// pageable memory with one 2-D copy runs at 194 GB/s, but device -> host
// 2-D copies into pageable memory ran at 1.2 GB/s; the rows are therefore
// first packed on the device (a device-to-device 2-D copy into a pool
// buffer) and read back with one 1-D copy.  (Staging through page-locked
// chunks, also measured, ran at the speed of the host memcpy: 17.5 GB/s.)
// ---------------------------------------------------------------------------
static MPStatus mp_copy_rows(bool h2d, void *dev_ptr, size_t pitch, void *host, size_t rowbytes, size_t rows,
                             cudaStream_t s)
{
    cudaError_t e;
    if (pitch == rowbytes) {
        e = cudaMemcpyAsync(h2d ? dev_ptr : host, h2d ? host : dev_ptr, rows * rowbytes,
                            h2d ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, s);
    } else if (h2d) {
        e = cudaMemcpy2DAsync(dev_ptr, pitch, host, rowbytes, rowbytes, rows, cudaMemcpyHostToDevice, s);
    } else {
        void *packed = nullptr;
        MPStatus st = mp_malloc_async(&packed, rows * rowbytes, s);
        if (st != MILLIPYDE_SUCCESS) return st;
        e = cudaMemcpy2DAsync(packed, rowbytes, dev_ptr, pitch, rowbytes, rows, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(host, packed, rows * rowbytes, cudaMemcpyDeviceToHost, s);
        mp_free_async(packed, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return mp_cuda_status(e);
}

extern "C" MPStatus mpobj_copy_from_host(MPObjData *obj, const void *host, int ndims,
                                         const int64_t *shape, int type, int itemsize,
                                         MPBool image)
{
    if (!obj || ndims < 0 || ndims > 32 || itemsize <= 0) return MP_ERROR_INVALID_ARGS;
    for (int i = 0; i < ndims; ++i)
        if (shape[i] < 0 || shape[i] > INT_MAX) return MP_ERROR_TOO_LARGE;
    int dev = mp_pick_device();
    if (dev < 0) return MP_ERROR_NO_DEVICE;
    MPStatus st = mp_device_setup(dev);
    if (st != MILLIPYDE_SUCCESS) return st;
    MP_CUDA_TRY(cudaSetDevice(dev));
    cudaStream_t s = mp_streams[dev];

    int *dims = (int *)malloc(sizeof(int) * 2 * (ndims > 0 ? ndims : 1));
    if (!dims) return MP_ERROR_OUT_OF_MEMORY;
    for (int i = 0; i < ndims; ++i) dims[i] = (int)shape[i];
    // C-contiguous strides
    size_t stride = (size_t)itemsize;
    for (int i = ndims - 1; i >= 0; --i) {
        if (stride > INT_MAX) { free(dims); return MP_ERROR_TOO_LARGE; }
        dims[ndims + i] = (int)stride;
        stride *= (size_t)shape[i];
    }
    size_t rows = ndims >= 1 ? (size_t)shape[0] : 1;
    size_t rowbytes = (size_t)itemsize;
    for (int i = 1; i < ndims; ++i) rowbytes *= (size_t)shape[i];
    size_t pitch = rowbytes;
    const bool pitched = image && (ndims == 2 || ndims == 3);
    if (pitched) {
        pitch = (rowbytes + 15) / 16 * 16;
        if (pitch > INT_MAX) { free(dims); return MP_ERROR_TOO_LARGE; }
        dims[ndims] = (int)pitch;
    }
    size_t nbytes = rows * pitch;
    void *d = nullptr;
    st = mp_malloc_async(&d, nbytes, s);
    if (st != MILLIPYDE_SUCCESS) { free(dims); return st; }
    if (nbytes) {
        st = mp_copy_rows(true, d, pitch, const_cast<void *>(host), rowbytes, rows, s);
        if (st != MILLIPYDE_SUCCESS) {
            mp_free_async(d, s);
            free(dims);
            return st;
        }
    }
    obj->device_data = d;
    obj->ndims = ndims;
    obj->dims = dims;
    obj->type = type;
    obj->mem_loc = dev;
    obj->stream = (void *)s;
    obj->pinned = MP_FALSE;
    obj->nbytes = nbytes;
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpobj_copy_to_host(const MPObjData *o, void *host)
{
    if (!o) return MP_ERROR_INVALID_ARGS;
    size_t total = mpobj_host_nbytes(o);
    if (total == 0) return MILLIPYDE_SUCCESS;
    if (!o->device_data) return MP_ERROR_NULL_DATA;
    MP_CUDA_TRY(cudaSetDevice(o->mem_loc));
    cudaStream_t s = (cudaStream_t)o->stream;
    size_t rows = o->ndims >= 1 ? (size_t)o->dims[0] : 1;
    size_t rowbytes = mp_row_bytes(o, mp_obj_itemsize(o));
    size_t pitch = o->ndims >= 2 ? (size_t)o->dims[o->ndims] : rowbytes;
    if (o->ndims < 2) rowbytes = total, rows = 1, pitch = total;
    MPStatus st = mp_copy_rows(false, o->device_data, pitch, host, rowbytes, rows, s);
    if (st != MILLIPYDE_SUCCESS) return st;
    return mp_check_device_error(s);
}

extern "C" MPObjData *mpobj_clone_data(const MPObjData *o, int device_id, int stream_id)
{
    (void)stream_id;
    if (!o) return nullptr;
    if (!mpdev_is_valid_device(device_id)) device_id = o->mem_loc;
    if (device_id != o->mem_loc) return nullptr;   // one GPU per process: no peer copies
    if (mp_device_setup(device_id) != MILLIPYDE_SUCCESS) return nullptr;
    if (cudaSetDevice(device_id) != cudaSuccess) return nullptr;
    MPObjData *c = (MPObjData *)malloc(sizeof(MPObjData));
    if (!c) return nullptr;
    *c = *o;
    c->pinned = MP_FALSE;
    c->stream = mp_streams[device_id];
    c->dims = (int *)malloc(sizeof(int) * 2 * (o->ndims > 0 ? o->ndims : 1));
    if (!c->dims) { free(c); return nullptr; }
    memcpy(c->dims, o->dims, sizeof(int) * 2 * o->ndims);
    c->device_data = nullptr;
    cudaStream_t s = (cudaStream_t)c->stream;
    if (o->nbytes) {
        if (mp_malloc_async(&c->device_data, o->nbytes, s) != MILLIPYDE_SUCCESS) {
            free(c->dims); free(c); return nullptr;
        }
        // order after any pending work on the source's stream
        if (o->stream != c->stream) cudaStreamSynchronize((cudaStream_t)o->stream);
        if (cudaMemcpyAsync(c->device_data, o->device_data, o->nbytes, cudaMemcpyDeviceToDevice, s) !=
            cudaSuccess) {
            mp_free_async(c->device_data, s); free(c->dims); free(c); return nullptr;
        }
    }
    return c;
}

extern "C" void mpobj_dealloc_device_data(MPObjData *o)
{
    if (!o) return;
    if (o->device_data) {
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(o->mem_loc);
        mp_free_async(o->device_data, (cudaStream_t)o->stream);
        cudaSetDevice(prev);
    }
    o->device_data = nullptr;
    if (o->dims) free(o->dims);
    o->dims = nullptr;
}

// ---------------------------------------------------------------------------
// Random numbers: a counter hashed by the SplitMix64 finaliser.
// ---------------------------------------------------------------------------
static inline uint64_t mp_mix64(uint64_t z)
{
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

extern "C" double mp_counter_uniform(uint64_t seed, uint64_t index, uint32_t stage, uint32_t slot)
{
    uint64_t h = mp_mix64(seed);
    h = mp_mix64(h ^ index);
    h = mp_mix64(h ^ (((uint64_t)stage << 32) | slot));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

static std::atomic<uint64_t> mp_rng_seed{0};
static std::atomic<uint64_t> mp_rng_counter{0};
static std::once_flag mp_rng_once;

static void mp_rng_init()
{
    std::call_once(mp_rng_once, []() {
        struct timespec ts;
        clock_gettime(CLOCK_REALTIME, &ts);
        uint64_t s = (uint64_t)ts.tv_nsec ^ ((uint64_t)ts.tv_sec << 30) ^ (uint64_t)(uintptr_t)&ts;
        if (mp_rng_seed.load() == 0) mp_rng_seed.store(mp_mix64(s));
    });
}

extern "C" void mp_seed(uint64_t seed)
{
    mp_rng_init();
    mp_rng_seed.store(seed);
    mp_rng_counter.store(0);
}

static double mp_next_uniform()
{
    mp_rng_init();
    uint64_t i = mp_rng_counter.fetch_add(1);
    return mp_counter_uniform(mp_rng_seed.load(), i, 0xFFFFFFFFu, 0);
}

extern "C" MPStatus random_double_in_range(double min, double max, double *result)
{
    if (!result) return MP_ERROR_INVALID_ARGS;
    *result = min + mp_next_uniform() * (max - min);
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus random_int_in_range(int min, int max, int *result)
{
    if (!result || max < min) return MP_ERROR_INVALID_ARGS;
    uint64_t span = (uint64_t)((int64_t)max - (int64_t)min + 1);
    uint64_t v = (uint64_t)(mp_next_uniform() * (double)span);
    if (v >= span) v = span - 1;
    *result = (int)((int64_t)min + (int64_t)v);
    return MILLIPYDE_SUCCESS;
}
