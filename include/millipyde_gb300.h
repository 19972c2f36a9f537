/*
 * millipyde_gb300.h -- C-ABI of the GB300 (sm_103a) image-operation library.
 *
 * This header is the drop-in boundary for millipyde's image hot path.  It
 * keeps the reference's object descriptor (MPObjData), its status codes, its
 * per-op argument structs and its per-op entry points (same names, same
 * MPFunc signature), so a build of the reference's CPython layer can link
 * against libmillipyde_gb300.so instead of src/millipyde_image.cpp.
 *
 * Everything is plain C: pointers, sizes and status codes.  No function
 * throws, none calls exit(); every failure is an MPStatus.  All entry points
 * are safe to call without the Python GIL and from several host threads
 * (per-call parameters travel as kernel arguments or in per-call device
 * tables; the one shared mutable device symbol is the scratch array and
 * error word of mpk_pipeline_run_noalloc, whose overlapping calls race).
 *
 * Reference interfaces replaced (paths within jasbury1/millipyde):
 *   src/include/millipyde.h:16-126      MPObjData, MPStatus, MPFunc, arg structs
 *   src/include/millipyde_image.h:18-48 mpimg_* entry points
 *   src/include/millipyde_objects.h     mpobj_* object memory
 *   src/include/millipyde_devices.h     mpdev_* (one-GPU subset)
 *   src/millipyde.c:8-173               mperr_str, random_*_in_range
 */
#ifndef MILLIPYDE_GB300_H
#define MILLIPYDE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MP_TRUE 1
#define MP_FALSE 0

/* Memory locations, as in src/include/millipyde.h:9-12. */
#define HOST_LOC -1
#define DEVICE_LOC_NO_AFFINITY -2

typedef int MPBool;

/*
 * Device object descriptor; same fields and order as the reference
 * (src/include/millipyde.h:16-25).
 *   dims     int[2*ndims]: shape, then byte strides.  For images (ndims 2 or
 *            3) dims[ndims] is the ROW PITCH in bytes.  Images allocated by
 *            this library have a pitch rounded up to 16 bytes so that every
 *            row start is a legal TMA address; dims[ndims+1] is the pixel
 *            stride (channels * itemsize).
 *   type     NumPy type number (NPY_FLOAT32 = 11, NPY_FLOAT64 = 12, ...).
 *   nbytes   size of the device allocation (rows * pitch for images).
 *   stream   cudaStream_t the object's work is ordered on.
 */
typedef struct {
    void *device_data;
    int ndims;
    int *dims;
    int type;
    int mem_loc;
    void *stream;
    MPBool pinned;
    size_t nbytes;
} MPObjData;

/*
 * Status codes.  The first block keeps the reference's names AND values
 * (src/include/millipyde.h:27-94); the second block is new: the reference
 * terminated the process on GPU errors (src/include/millipyde_hip_util.h:7-16)
 * and silently returned success on unsupported inputs.
 */
typedef enum mp_status_codes {
    MILLIPYDE_SUCCESS = 0,

    MOD_ERROR,
    MOD_ERROR_CREATE_GPUARRAY_TYPE,
    MOD_ERROR_CREATE_GPUIMAGE_TYPE,
    MOD_ERROR_CREATE_OPERATION_TYPE,
    MOD_ERROR_CREATE_PIPELINE_TYPE,
    MOD_ERROR_CREATE_DEVICE_TYPE,
    MOD_ERROR_CREATE_GENERATOR_TYPE,
    MOD_ERROR_ADD_GPUARRAY,
    MOD_ERROR_ADD_GPUIMAGE,
    MOD_ERROR_ADD_OPERATION,
    MOD_ERROR_ADD_PIPELINE,
    MOD_ERROR_ADD_DEVICE,
    MOD_ERROR_ADD_GENERATOR,

    DEV_ERROR_CURRENT_DEVICE,
    DEV_ERROR_DEVICE_COUNT,
    DEV_ERROR_DEVICE_PROPERTIES,
    DEV_ERROR_PEER_ACCESS_MATRIX_ALLOC,
    DEV_ERROR_DEVICE_ARRAY_ALLOC,
    DEV_WARN_NO_PEER_ACCESS,
    DEV_WARN_BAD_DEVICE,

    WORK_ERROR_INIT_PTHREAD,
    WORK_ERROR_INIT_COND,
    WORK_ERROR_INIT_MUX,
    WORK_ERROR_ALLOC_WORK_POOL,
    WORK_ERROR_ALLOC_WORK_NODE,
    WORK_ERROR_NULL_WORK_POOL,

    TYPE_ERROR_NON_GPUOBJ,

    RAND_ERROR_INSUFFICIENT_BYTES,

    GPUARRAY_ERROR_CONSTRUCTION_WITHOUT_ARRAY_TYPE,
    GPUARRAY_ERROR_CONSTRUCTION_WITHOUT_NUMERIC_ARRAY,

    GPUIMAGE_ERROR_CONSTRUCTION_WITHOUT_ARRAY_TYPE,
    GPUIMAGE_ERROR_CONSTRUCTION_WITHOUT_IMAGE_FORMAT,
    GPUIMAGE_ERROR_CONSTRUCTION_WITHOUT_IMAGE_DIMS,

    GPUOPERATION_ERROR_CONSTRUCTION_NO_ARGS,
    GPUOPERATION_ERROR_INVALID_PROBABILITY,
    GPUOPERATION_ERROR_CONSTRUCTION_NAMED_ARGS,
    GPUOPERATION_ERROR_RUN_WITHOUT_STRING_METHOD,
    GPUOPERATION_ERROR_RUN_UNKNOWN_STRING_METHOD,
    GPUOPERATION_ERROR_RUN_NO_DEV_RANDOM,
    GPUOPERATION_ERROR_RUN_CANNOT_READ_DEV_RANDOM,

    GPUPIPELINE_ERROR_CONSTRUCTION_INVALID_ARGS,
    GPUPIPELINE_ERROR_INVALID_DEVICE,
    GPUPIPELINE_ERROR_UNUSABLE_DEVICE,
    GPUPIPELINE_ERROR_CONSTRUCTION_NAMED_ARGS,
    GPUPIPELINE_ERROR_NONLIST_INPUTS,
    GPUPIPELINE_ERROR_NONLIST_OPERATIONS,
    GPUPIPELINE_ERROR_NONGPU_INPUT,

    GPUGENERATOR_ERROR_INVALID_DEVICE,
    GPUGENERATOR_ERROR_INVALID_MAX,
    GPUGENERATOR_ERROR_INVALID_RETURN_TO,
    GPUGENERATOR_ERROR_UNUSABLE_DEVICE,
    GPUGENERATOR_ERROR_CONSTRUCTION_NAMED_ARGS,
    GPUGENERATOR_ERROR_INVALID_INPUT,
    GPUGENERATOR_ERROR_NONLIST_OPERATIONS,

    /* ---- added by this library ---- */
    MP_ERROR_NO_DEVICE = 1000,     /* no CUDA device (or no driver) */
    MP_ERROR_CUDA,                 /* a CUDA runtime call failed; see mp_last_cuda_error() */
    MP_ERROR_OUT_OF_MEMORY,        /* device allocation failed */
    MP_ERROR_INVALID_ARGS,         /* bad scalar argument (sigma <= 0, NaN, ...) */
    MP_ERROR_UNSUPPORTED_TYPE,     /* dtype/channel layout this op does not handle */
    MP_ERROR_UNSUPPORTED_DIMS,     /* bad rank / zero-size / too-large image */
    MP_ERROR_NULL_DATA,            /* descriptor without device data */
    MP_ERROR_KERNEL_TIMEOUT,       /* a bounded device-side wait gave up */
    MP_ERROR_BAD_DESCRIPTOR,       /* malformed batch descriptor (checked on the host) */
    MP_ERROR_TOO_LARGE             /* request above a documented limit */
} MPStatus;

/* Per-op entry point signature (src/include/millipyde.h:96). */
typedef MPStatus (*MPFunc)(MPObjData *, void *);

typedef struct {
    MPFunc func;
    MPObjData *obj_data;
    void *args;
    double probability;
} MPRunnable;

/* Argument structs, src/include/millipyde.h:105-126. */
typedef struct { double angle; } RotateArgs;          /* degrees */
typedef struct { double sigma; } GaussianArgs;
typedef struct { double delta; } BrightnessArgs;
typedef struct { double r_mult; double g_mult; double b_mult; } ColorizeArgs;
typedef struct { double gamma; double gain; } GammaArgs;

/* src/millipyde.c:8-138. */
const char *mperr_str(MPStatus status);

/* Text of the last CUDA error seen by the calling thread (or ""). */
const char *mp_last_cuda_error(void);

/*
 * Random draws, src/millipyde.c:140-173.  The reference read getrandom() and
 * could not be seeded; these draw from a process-wide counter-based stream
 * (SplitMix64 finaliser over a 64-bit counter) that mp_seed() resets, so a
 * seeded run is reproducible.
 */
MPStatus random_int_in_range(int min, int max, int *result);
MPStatus random_double_in_range(double min, double max, double *result);
void mp_seed(uint64_t seed);
/* Pure counter draw: uniform double in [0,1) for (seed, index, stage, slot). */
double mp_counter_uniform(uint64_t seed, uint64_t index, uint32_t stage, uint32_t slot);

/* ------------------------------------------------------------------------ */
/* Per-op entry points, src/include/millipyde_image.h:18-48 and             */
/* src/millipyde_image.cpp:530-717.  Each mutates obj_data in place (new     */
/* device buffer, dims/strides/type/nbytes updated) and is stream-ordered on */
/* obj_data->stream.  float32 images (type 11) with 1, 3 or 4 channels use   */
/* the float path: values in [0,1], FP32 arithmetic.  uint8 RGBA (type 2,    */
/* 4 channels) and float64 greyscale (type 12, 2-D) use the reference's own  */
/* arithmetic ("legacy" path).                                               */
/* ------------------------------------------------------------------------ */
MPStatus mpimg_color_to_greyscale(MPObjData *obj_data, void *args);  /* args unused */
MPStatus mpimg_transpose(MPObjData *obj_data, void *args);           /* args unused */
MPStatus mpimg_gaussian(MPObjData *obj_data, void *args);            /* GaussianArgs */
MPStatus mpimg_fliplr(MPObjData *obj_data, void *args);              /* args unused */
MPStatus mpimg_rotate(MPObjData *obj_data, void *args);              /* RotateArgs */
MPStatus mpimg_brightness(MPObjData *obj_data, void *args);          /* BrightnessArgs */
MPStatus mpimg_colorize(MPObjData *obj_data, void *args);            /* ColorizeArgs */
MPStatus mpimg_adjust_gamma(MPObjData *obj_data, void *args);        /* GammaArgs */

/* ------------------------------------------------------------------------ */
/* Object memory: replaces src/millipyde_objects.cpp:18-120.                */
/* ------------------------------------------------------------------------ */

/* Copy a C-contiguous host array to the device.  For images (image != 0,
 * ndims 2 or 3) rows are stored with a 16-byte-aligned pitch.  obj_data->dims
 * is allocated with malloc (2*ndims ints) and owned by obj_data. */
MPStatus mpobj_copy_from_host(MPObjData *obj_data, const void *host, int ndims,
                              const int64_t *shape, int type, int itemsize,
                              MPBool image);
/* Bytes of the packed host copy (product of shape * itemsize). */
size_t mpobj_host_nbytes(const MPObjData *obj_data);
/* Copy to a packed host buffer of mpobj_host_nbytes() bytes (synchronous). */
MPStatus mpobj_copy_to_host(const MPObjData *obj_data, void *host);
/* Deep copy into a fresh descriptor (malloc'd).  NULL on failure. */
MPObjData *mpobj_clone_data(const MPObjData *obj_data, int device_id, int stream_id);
/* Free device data (stream-ordered) and the dims array; not the struct. */
void mpobj_dealloc_device_data(MPObjData *obj_data);
/* Item size in bytes for a NumPy type number, 0 if unknown. */
int mp_type_itemsize(int type);

/* ------------------------------------------------------------------------ */
/* Device layer: one-GPU subset of src/include/millipyde_devices.h.         */
/* ------------------------------------------------------------------------ */
MPStatus mpdev_initialize(void);
int mpdev_get_device_count(void);
int mpdev_get_recommended_device(void);
int mpdev_get_target_device(void);
void mpdev_set_target_device(int device_id);
MPBool mpdev_is_valid_device(int device_id);
void *mpdev_get_stream(int device_id, int stream_id);
MPStatus mpdev_synchronize(void);
/* Device name (e.g. "NVIDIA GB300") into buf (len bytes, NUL-terminated). */
MPStatus mpdev_get_device_name(int device_id, char *buf, int len);
MPStatus mpdev_stream_synchronize(void *stream);
/* Reserved and in-use bytes of the device's stream-ordered memory pool (the
 * pool every allocation of this library comes from), and the in-use high
 * water mark since the last mpdev_pool_reset_peak (used_peak may be null). */
MPStatus mpdev_pool_usage(int device_id, uint64_t *reserved, uint64_t *used, uint64_t *used_peak);
MPStatus mpdev_pool_reset_peak(int device_id);
/* Failure injection on the host: every later device allocation of the
 * library larger than max_request_bytes fails with MP_ERROR_OUT_OF_MEMORY
 * as if the device were full (0 removes the limit).  The reference exited
 * the process on a failed hipMalloc (src/include/millipyde_hip_util.h:7-16);
 * here the failing call returns the status and leaves its object as it was. */
void mpdev_set_alloc_limit(size_t max_request_bytes);
/* Self-test of the bounded device-side waits every kernel uses: one CTA
 * waits on a barrier phase that never completes, gives up after `polls`
 * polls (1 .. 2^21; about 1 us each after the first 2048) and reports it.
 * Returns MP_ERROR_KERNEL_TIMEOUT with the device's error word cleared again,
 * the context still usable. */
MPStatus mpdev_selftest_wait_timeout(uint32_t polls, void *stream);

/* ------------------------------------------------------------------------ */
/* Batch pipeline: the fused, ragged path behind Pipeline.run and           */
/* Generator (src/gpupipeline.c:233-403, src/gpugenerator.c:202-281).       */
/* ------------------------------------------------------------------------ */
typedef enum {
    MP_OP_NONE = 0,
    MP_OP_RGB2GREY = 1,
    MP_OP_TRANSPOSE = 2,
    MP_OP_GAUSSIAN = 3,     /* p0 = sigma */
    MP_OP_FLIPLR = 4,
    MP_OP_ROTATE = 5,       /* p0 = angle in degrees */
    MP_OP_BRIGHTNESS = 6,   /* p0 = delta */
    MP_OP_ADJUST_GAMMA = 7, /* p0 = gamma, p1 = gain */
    MP_OP_COLORIZE = 8      /* p0,p1,p2 = r,g,b multipliers */
} MPOpCode;

/* One pipeline stage.  When `random` is set each parameter k is drawn per
 * image as lo[k] + u*(hi[k]-lo[k]) with u = mp_counter_uniform(seed, index,
 * stage, k); otherwise lo[] holds the fixed values.  probability in (0,1)
 * applies the stage to an image iff mp_counter_uniform(seed, index, stage, 3)
 * <= probability (src/gpuoperation.c:186-210); other values mean "always". */
typedef struct {
    int op;
    int random;
    double lo[3];
    double hi[3];
    double probability;
} MPStage;

/* A float32 image in device memory: `channels` interleaved floats per pixel,
 * rows `pitch` bytes apart (pitch a multiple of 4; a multiple of 16 enables
 * the TMA load path). */
typedef struct {
    void *data;
    int height;
    int width;
    int channels;
    int pitch;
} MPImage;

/* Largest gaussian radius the kernels accept; radius = ceil(3*sigma). */
#define MP_MAX_RADIUS 48

/* Fill out[i].height/width/channels/pitch (pitch rounded up to 16 bytes;
 * data left untouched) for the result of running the stages on in[i]. */
MPStatus mpk_pipeline_shapes(const MPStage *stages, int nstages, const MPImage *in,
                             MPImage *out, int nimgs, uint64_t seed, uint64_t index0);

/* Run the stages on nimgs images: in[i] -> out[i] (out[i] from
 * mpk_pipeline_shapes, with data set; in and out must not overlap).  Image i
 * draws its random parameters with index = index0 + i.  Stream-ordered;
 * temporary buffers come from the device's stream-ordered pool. */
MPStatus mpk_pipeline_run(const MPStage *stages, int nstages, const MPImage *in,
                          MPImage *out, int nimgs, uint64_t seed, uint64_t index0,
                          void *stream);

/* Same, but forces one launch per stage and image (the plain per-op kernels)
 * instead of the fused segments; used as the unfused baseline. */
MPStatus mpk_pipeline_run_unfused(const MPStage *stages, int nstages, const MPImage *in,
                                  MPImage *out, int nimgs, uint64_t seed, uint64_t index0,
                                  void *stream);

/* Plans: resolve parameters, segment and upload the job tables once, then
 * launch (kernel launches only, so mpk_plan_launch can be captured into a
 * CUDA graph and replayed).  The images and buffers named at creation must
 * stay valid while the plan is used. */
typedef struct MPPlan MPPlan;
MPStatus mpk_plan_create(const MPStage *stages, int nstages, const MPImage *in, const MPImage *out,
                         int nimgs, uint64_t seed, uint64_t index0, void *stream, MPPlan **plan);
MPStatus mpk_plan_launch(MPPlan *plan, void *stream);
int mpk_plan_num_launches(const MPPlan *plan);
MPStatus mpk_plan_destroy(MPPlan *plan);

/* Launches launches [first, first+count) of a plan only, and describes
 * launch i (kind: 0 pointwise, 1 gaussian, 2 rotate, 3 transpose,
 * 4 streaming gaussian, 5 footprint-staged rotate, 8 streaming gaussian
 * (register-window family), 9 gaussian and rotate fused; njobs
 * images; tiles CTAs; bytes = algorithmic bytes moved: every input pixel read
 * once and every output pixel written once, float32). */
MPStatus mpk_plan_launch_range(MPPlan *plan, int first, int count, void *stream);
MPStatus mpk_plan_launch_info(const MPPlan *plan, int i, int *kind, int *njobs, int *tiles,
                              double *bytes);

/* Host-buffer batch: in[i].data / out[i].data are HOST pointers and pitch the
 * host row stride in bytes (out[i] geometry from mpk_pipeline_shapes, pitch
 * may be changed to the packed row size).  Images move in chunks through
 * device staging buffers: the host->device copy of chunk k+1, the kernels of
 * chunk k and the device->host copy of chunk k-1 run concurrently on three
 * streams.  Page-locked host memory (cudaHostAlloc / cudaHostRegister) gives
 * the overlap; pageable memory works but serialises the copies.  Returns
 * after the last result is on the host. */
MPStatus mpk_pipeline_run_host(const MPStage *stages, int nstages, const MPImage *in,
                               const MPImage *out, int nimgs, uint64_t seed, uint64_t index0,
                               void *stream);

/* Autotuning: tile size (tw x th output pixels, multiples of 8) of the
 * gaussian kernel for a channel variant (source channels, channels after the
 * prologue), prologue flag and radius range; the planner prefers these over
 * its built-in table.  millipyde_gb300/autotune.py times candidates on the
 * device and records the fastest.  get returns what the planner would use. */
MPStatus mpk_tune_set_gauss_tile(int cin, int cmid, int has_pro, int radius_lo, int radius_hi,
                                 int tw, int th);
MPStatus mpk_tune_get_gauss_tile(int cin, int cmid, int has_pro, int radius, int *tw, int *th);
/* TMA stage count (2..6) of the streaming gaussian for a channel count
 * after the prologue (1, 3 or 4). */
MPStatus mpk_tune_set_stream(int cmid, int stages);
/* Intermediate bytes one chunk of a fused batch may hold (at least 1 MB;
 * default 2 GB): a batch runs as one launch per segment per chunk. */
MPStatus mpk_tune_set_chunk_bytes(size_t bytes);
/* Geometry of the persistent kernels, per launch kind (5 footprint rotate,
 * 8 streaming gaussian, 9 fused gaussian + rotate); value 0 restores the
 * built-in choice.  param 0: work items per resident CTA of a streaming
 * gaussian launch (rows per item follow; kind 8 only, 1..64); param 1: cap
 * on resident CTAs per SM (1..32); param 2: cap on the streaming gaussian's
 * strip width in columns (kind 8 only, a multiple of 8 from 64).  Set by
 * millipyde_gb300/autotune.py from timings; plans created afterwards follow
 * it. */
MPStatus mpk_tune_set_kernel(int kind, int param, int value);
MPStatus mpk_tune_get_kernel(int kind, int param, int *value);
/* Fusion of a one-channel gaussian (radius <= 12; 1-channel source, or a
 * 3-channel source whose prologue ends in rgb2grey) with the rotate after
 * it into one kernel that keeps the blurred image in shared memory:
 * 1 = on, 0 = off (the default: two launches and an intermediate in HBM).
 * The autotuner times both and records the faster.  Plans created
 * afterwards follow the setting. */
MPStatus mpk_tune_set_fuse(int enable);
/* Clears the tuned tables and restores the defaults (fusion off). */
void mpk_tune_clear(void);

/* Differentiable chains on dense batches (the autograd path): B images of
 * H x W x C float32, packed rows, image b at x + b*H*W*C; ops[nops] MPOpCode;
 * params[(b*nops + k)*3 + j] explicit per-image parameters (host memory).
 * forward writes y (geometry from mpk_chain_shape); backward recomputes the
 * forward intermediates in image chunks, writes dx and ADDS parameter
 * gradients (FP64) to dparams[(b*nops + k)*3 + j] (device memory, zeroed by
 * the caller). */
MPStatus mpk_chain_shape(const int *ops, int nops, int H, int W, int C, int *Ho, int *Wo, int *Co);
MPStatus mpk_chain_forward(const int *ops, int nops, const double *params, const float *x, float *y,
                           int B, int H, int W, int C, void *stream);
MPStatus mpk_chain_backward(const int *ops, int nops, const double *params, const float *x,
                            const float *dy, float *dx, double *dparams, int B, int H, int W, int C,
                            void *stream);
/* The same with param_mask[k] != 0 for every op k whose parameters want a
 * gradient (null: all of them); ops whose mask is 0 skip their parameter
 * passes (a gaussian's two d sigma passes). */
MPStatus mpk_chain_backward_masked(const int *ops, int nops, const double *params, const float *x,
                                   const float *dy, float *dx, double *dparams, const int *param_mask,
                                   int B, int H, int W, int C, void *stream);
/* Saved forward intermediates: the forward plan writes the input a_k of
 * every op k that opens one of its later segments anyway; with a saved
 * block the forward writes them there and the backward reads them instead
 * of recomputing them (it recomputes only the intermediates it needs that
 * were not saved, starting from the nearest saved one).  Layout for B
 * images: *count entries (at most nops); entry s is a_{op_index[s]}, B dense
 * images (rows of w*c floats, shape from the chain) from byte offset[s];
 * *bytes is the whole block (0: nothing is saved for this chain).  The
 * layout depends on the op kinds and shapes only.  op_index / offset may
 * be null.  The block must stay untouched between the two calls. */
MPStatus mpk_chain_saved_layout(const int *ops, int nops, int B, int H, int W, int C, int *count,
                                int *op_index, size_t *offset, size_t *bytes);
MPStatus mpk_chain_forward_saved(const int *ops, int nops, const double *params, const float *x, float *y,
                                 void *saved, int B, int H, int W, int C, void *stream);
/* y (may be null) is the forward's output, unmodified: a chain that ends
 * in a lone brightness back-propagates it from y (clamp01(a + delta) lies
 * strictly inside (0, 1) exactly when a + delta does), so its input is
 * neither saved nor recomputed. */
MPStatus mpk_chain_backward_saved(const int *ops, int nops, const double *params, const float *x,
                                  const void *saved, const float *y, const float *dy, float *dx,
                                  double *dparams, const int *param_mask, int B, int H, int W, int C,
                                  void *stream);

/* Allocation-free batch.  No counterpart in the reference.  For callers that
 * cannot allocate device memory (GPU memory owned by another allocator or
 * reserved up front, or a loop where a cudaMalloc would stall): the same
 * stages as mpk_pipeline_run on caller-provided device buffers (in[i] ->
 * out[i], geometry from mpk_pipeline_shapes), allocating no device memory:
 * no cudaMalloc, no cudaFree, no device-allocating library routine (job
 * descriptors travel as kernel parameters).  Intermediates live in a 32 MB
 * file-scope device array (two 16 MB halves) that every GPU loading the
 * library holds until exit; any image whose intermediate would exceed 16 MB
 * is rejected with MP_ERROR_TOO_LARGE before anything is launched.  Images
 * run one after another on `stream`; the call returns when they are done.
 * Every image is validated (descriptors, parameters, intermediate sizes)
 * before the first launch, so a rejected call leaves every output untouched.
 * Its first call on a device resolves the array's device address (set-up,
 * with that device current; make that first call before any stream capture);
 * the address is kept for the life of the process, so cudaDeviceReset ends
 * this entry point's use in that process.  Every call uses the same array and
 * error word, so calls that overlap on the GPU (other threads or streams)
 * race; each call clears the error word before its first launch, and stale
 * array contents from an earlier call are never read. */
MPStatus mpk_pipeline_run_noalloc(const MPStage *stages, int nstages, const MPImage *in,
                                  const MPImage *out, int nimgs, uint64_t seed, uint64_t index0,
                                  void *stream);

/* Object-level batch used by Pipeline.run: applies the stages in place to
 * each object (float32 images: fused path when fused != 0, else one launch
 * per stage and image; other dtypes: the per-op entry points).  Image i uses
 * index0 + i for its random draws; an object listed twice is processed twice,
 * in list order. */
MPStatus mpk_pipeline_run_objects(const MPStage *stages, int nstages, MPObjData **objs, int nobjs,
                                  uint64_t seed, uint64_t index0, int fused);
/* Object-level batch used by Generator: outs[i] (zeroed structs owned by the
 * caller) receive new device objects holding the stages applied to srcs[i];
 * srcs are not modified. */
MPStatus mpk_pipeline_produce(const MPStage *stages, int nstages, MPObjData **srcs,
                              MPObjData **outs, int n, uint64_t seed, uint64_t index0);

/* Per-image parameters the pipeline resolved: params[(i*nstages+s)*4 + k],
 * k = 0..2 the op parameters, k = 3 is 1.0 when the stage ran, else 0.0. */
MPStatus mpk_pipeline_resolve(const MPStage *stages, int nstages, int nimgs,
                              uint64_t seed, uint64_t index0, double *params);

#ifdef __cplusplus
}
#endif

#endif /* MILLIPYDE_GB300_H */
