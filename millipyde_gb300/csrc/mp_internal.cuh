// mp_internal.cuh -- shared definitions of the CUDA side of millipyde_gb300.
//
// Kernel descriptors (MPJob), the pointwise-op interpreter used as prologue /
// epilogue of every kernel kind, and the inline-PTX wrappers for mbarrier and
// TMA (cp.async.bulk.tensor) used by the gaussian kernel.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/millipyde_gb300.h"

// ---------------------------------------------------------------------------
// Limits
// ---------------------------------------------------------------------------
#define MP_MAX_PW 8                       // pointwise ops in one prologue/epilogue
// Internal op of the pointwise adjoint: brightness back-propagated from its
// OUTPUT v = clamp01(x + delta).  v lies strictly inside (0, 1) exactly when
// x + delta does, so the gradient mask (and d delta) needs no x.
#define MP_OP_BRIGHTNESS_OUT 64
#define MP_MAX_TAPS (2 * MP_MAX_RADIUS + 1)
#define MP_FIX_FRAC 40                    // fractional bits of rotate coordinates
#define MP_SPIN_FAST 2048                 // try_wait polls before backing off
#define MP_SPIN_LIMIT (1u << 21)          // bounded wait: ~2 s with 1 us backoff

// Segment kernel kinds.  GSTREAM is the strip-streaming gaussian
// (mp_stream.cu), used for GAUSS segments whose source rows are TMA-legal and
// whose epilogue is per-channel.
// RSTREAM is the footprint-staged rotate (mp_rot.cu), used for ROTATE
// segments without a prologue whose source rows are TMA-legal.
// VH is the streaming gaussian of mp_vh.cuh (single-channel and
// channel-preserving families), for radii up to MP_VH_RMAX.
// RADJ / RDTH are the rotate adjoint's dx = R^T g and d theta passes on the
// footprint-staged kernel (variant = 8 * mode + channels).
// FUSE is a one-channel gaussian followed by a rotate in one kernel, the
// blurred image kept in shared memory (mp_fuse.cuh).
enum MPKind {
    MPK_POINT = 0, MPK_GAUSS = 1, MPK_ROTATE = 2, MPK_TRANSPOSE = 3, MPK_GSTREAM = 4, MPK_RSTREAM = 5,
    MPK_RADJ = 6, MPK_RDTH = 7, MPK_VH = 8, MPK_FUSE = 9
};
#define MP_VH_RMAX 12
#define MP_VH_RBIG 24   // largest bucket radius of the mp_vh.cuh kernels


// Output tile of the footprint-staged rotate per channel count.
__host__ __device__ constexpr int mp_ro_tw(int c) { return c == 1 ? 64 : 32; }
__host__ __device__ constexpr int mp_ro_th(int c) { return c == 1 ? 64 : 32; }
#define MP_RO_NT 256
#define MP_RO_NT_WS (MP_RO_NT + 32)    // rotate and its dx: sampling threads + a producer warp

// ---------------------------------------------------------------------------
// Streaming gaussian geometry (host and device agree on it).  Rows are
// processed in blocks of MP_GS_RB; sizes in floats unless noted.  The strip
// width and CTA size are fixed per channel count after the prologue (cmid),
// and radii are rounded up to a compiled bucket (exact up to 12, then 16 and
// 24; larger radii run a loop over the taps).
// ---------------------------------------------------------------------------
#define MP_GS_MAXNS 6

// strip width, rows per block and CTA size per channel count after the prologue
__host__ __device__ constexpr int mp_gs_sw(int cmid) { return 64; }
__host__ __device__ constexpr int mp_gs_rb(int cmid) { return cmid == 1 ? 16 : 8; }
__host__ __device__ constexpr int mp_gs_nt(int cmid) { return cmid == 1 ? 128 : 64 * cmid; }
__host__ __device__ constexpr int mp_gs_bucket(int r) { return r <= 12 ? r : (r <= 16 ? 16 : (r <= 24 ? 24 : r)); }

struct GsGeom {
    int SW, lgSW;     // strip width in output pixels (power of two)
    int NS;           // TMA stages in the ring
    int BOXW;         // floats per TMA box row (48 for 3 source channels, else 64)
    int BOXS;         // floats from one box of a stage to the next
    int STG;          // floats per stage
    int GW;           // row stride of the channel planes G
    int HW;           // row stride of the horizontal-pass ring H (SW + 4)
    int HR;           // rows of H per channel (ring + mirrored head + read-ahead)
    int offS, offG, offH;   // byte offsets from the 128-byte aligned base
    int total;              // bytes (without alignment slack)
};

__host__ __device__ __forceinline__ int mp_gs_boxw(int cin) { return cin == 3 ? 48 : 64; }

// Geometry for ns stages and largest bucket radius rb over the launch.
// Radii outside the compiled buckets run loop passes that read up to 8 rows
// past the vertical window, so the H ring always carries 8 spare rows.
__host__ __device__ __forceinline__ GsGeom mp_gs_geom(int ns, int rb, int cin, int cmid)
{
    GsGeom g;
    const int sw = mp_gs_sw(cmid), RB = mp_gs_rb(cmid);
    g.SW = sw;
    g.lgSW = 0;
    while ((1 << g.lgSW) < sw) ++g.lgSW;
    g.NS = ns;
    g.BOXW = mp_gs_boxw(cin);
    const int R4 = (rb + 3) & ~3;
    const int GL = (sw + 2 * R4 + 4 + 15) & ~15;           // pixels per G row
    const int nbx = (GL * cin + g.BOXW - 1) / g.BOXW;
    g.BOXS = g.BOXW * RB + 32;                             // +128 B: box starts stay 128-B aligned
    g.STG = nbx * g.BOXS;
    g.GW = ((GL + 31) & ~31) + 4;                          // = 4 (mod 32): conflict-free column reads
    g.HW = sw + 4;
    const int L = (2 * rb + RB - 1) / RB;
    g.HR = (L + 1) * RB + 2 * rb + 8;
    g.offS = 1152;                                         // barriers + two 128-float tap arrays
    g.offG = g.offS + ns * g.STG * 4;
    g.offH = g.offG + cmid * RB * g.GW * 4;
    g.total = g.offH + cmid * g.HR * g.HW * 4;
    return g;
}

// Device-side error word values (written by kernels, read by the host).
enum { MP_KERR_NONE = 0, MP_KERR_TIMEOUT = 1 };

struct PwOp {
    int op;        // MP_OP_RGB2GREY / BRIGHTNESS / ADJUST_GAMMA / COLORIZE
    float p0, p1, p2;
};

struct PwList {
    int n;
    PwOp op[MP_MAX_PW];
};

// One image's work for one segment kernel.  The tensor map member makes the
// struct 128-byte aligned, so every entry of a job table in global memory
// holds a legal TMA descriptor address.
struct MPJob {
    CUtensorMap tmap;          // GAUSS: 2-D map over the source, box {64, th + 2r}
    const float *src;
    float *dst;
    long long cosq, sinq;      // ROTATE: cos/sin * 2^(MP_FIX_FRAC-1), rounded
    int h, w;                  // source height/width (pixels)
    int ho, wo;                // output height/width
    int src_pitch, dst_pitch;  // row pitches in floats
    int cin, cmid, cout;       // channels: source, after prologue, after epilogue
    int flip;                  // output map: mirror x (fliplr)
    int radius;                // GAUSS radius
    int tw, th;                // tile size (pixels)
    int tiles_x;               // tiles across this image
    int tile0;                 // first global tile index of this image
    int ntiles;                // tiles of this image
    int use_tma;               // GAUSS: source rows 16-byte aligned -> TMA path
    PwList pro, epi;
    float wts[MP_MAX_TAPS];    // GAUSS: normalised taps w[0..2r] (vertical pass)
    // ---- adjoint / reduction modes (zero for plain forward jobs)
    int hsep;                  // GAUSS: horizontal pass uses wts_h instead of wts
    int dot;                   // GAUSS: accumulate sum(out * aux) into acc[0], write nothing
    const float *aux;          // dot source (GAUSS) / output-space gradient (adjoints)
    int aux_pitch;             // in floats
    double *acc;               // per-image accumulators (parameter gradients)
    int pw_slot[MP_MAX_PW];    // POINT adjoint: acc slot (x3) of each pointwise op
    float cth, sth;            // ROTATE adjoint: cos/sin of the angle
    float wts_h[MP_MAX_TAPS];  // GAUSS: horizontal taps when hsep
    int vec_out;               // GSTREAM: destination rows 16-byte aligned (vector stores)
    int bxw, byh;              // RSTREAM: footprint box (floats per row, rows); FUSE: pixels
    PwList epi2;               // FUSE: the gaussian's epilogue (applied before the rotate)
};

// Shared-memory geometry (floats) of a FUSE launch, sized for its largest
// job: one chunk stage of the staged source region, the row pitch of the
// blur planes (= 4 mod 16) and the offset of the plane G from the base.
struct FzGeom {
    int stage;
    int gp;
    int offG;
};

// ---------------------------------------------------------------------------
// Pointwise ops.  Semantics follow the reference's per-pixel formulas
// (src/millipyde_image.cpp:64 grey, :392-394 brightness, :447-452 gamma,
// :494-524 colorize), in float32 on values in [0,1]; alpha (channel 3 of a
// 4-channel pixel) is left untouched as in the reference's RGBA kernels.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float mp_clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// One pointwise op on v[0..c-1]; returns the new channel count.
__device__ __forceinline__ int mp_pw_op(int op, float p0, float p1, float p2, float v[4], int c)
{
    const int cc = (c == 4) ? 3 : c;     // colour channels
    switch (op) {
    case MP_OP_RGB2GREY:
        if (c >= 3) {
            v[0] = fminf(1.0f, 0.2125f * v[0] + 0.7154f * v[1] + 0.0721f * v[2]);
            c = 1;
        }
        break;
    case MP_OP_BRIGHTNESS:
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (k < cc) v[k] = mp_clamp01(v[k] + p0);
        break;
    case MP_OP_ADJUST_GAMMA:
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (k < cc) v[k] = mp_clamp01(p1 * __powf(v[k], p0));
        break;
    case MP_OP_COLORIZE:
        if (c >= 3) {
            v[0] = fminf(1.0f, v[0] * p0);
            v[1] = fminf(1.0f, v[1] * p1);
            v[2] = fminf(1.0f, v[2] * p2);
        }
        break;
    default:
        break;
    }
    return c;
}

// Applies L to v[0..c-1] and returns the new channel count.
__device__ __forceinline__ int mp_pw_apply(const PwList &L, float v[4], int c)
{
    for (int i = 0; i < L.n; ++i) {
        const PwOp o = L.op[i];
        c = mp_pw_op(o.op, o.p0, o.p1, o.p2, v, c);
    }
    return c;
}

// A pointwise list with its first op held in registers: lists of one op (the
// common prologue / epilogue) run without reading the list per pixel.
struct PwFast {
    int n, op;
    float p0, p1, p2;
};

__device__ __forceinline__ PwFast mp_pw_fast(const PwList &L)
{
    PwFast f;
    f.n = L.n;
    f.op = L.n ? L.op[0].op : 0;
    f.p0 = L.n ? L.op[0].p0 : 0.f;
    f.p1 = L.n ? L.op[0].p1 : 0.f;
    f.p2 = L.n ? L.op[0].p2 : 0.f;
    return f;
}

__device__ __forceinline__ int mp_pw_apply_f(const PwFast &f, const PwList &L, float v[4], int c)
{
    if (f.n == 0) return c;
    if (f.n == 1) return mp_pw_op(f.op, f.p0, f.p1, f.p2, v, c);
    return mp_pw_apply(L, v, c);
}

// One channel-preserving pointwise op on a single value of channel c of a
// cm-channel pixel: the same arithmetic as mp_pw_op, one channel at a time
// (rgb2grey mixes channels and is never applied this way).
__device__ __forceinline__ float mp_pw_chan(int op, float p0, float p1, float p2, float v, int c, int cm)
{
    const bool colour = !(cm == 4 && c == 3);
    switch (op) {
    case MP_OP_BRIGHTNESS: return colour ? mp_clamp01(v + p0) : v;
    case MP_OP_ADJUST_GAMMA: return colour ? mp_clamp01(p1 * __powf(v, p0)) : v;
    case MP_OP_COLORIZE:
        if (cm >= 3 && c < 3) return fminf(1.0f, v * (c == 0 ? p0 : (c == 1 ? p1 : p2)));
        return v;
    default: return v;
    }
}

__device__ __forceinline__ float mp_pw_chan_f(const PwFast &f, const PwList &L, float v, int c, int cm)
{
    if (f.n == 0) return v;
    if (f.n == 1) return mp_pw_chan(f.op, f.p0, f.p1, f.p2, v, c, cm);
    for (int i = 0; i < L.n; ++i) v = mp_pw_chan(L.op[i].op, L.op[i].p0, L.op[i].p1, L.op[i].p2, v, c, cm);
    return v;
}

// Up to three channel-preserving pointwise ops held in registers, applied to
// N values at once (value k belongs to channel ch[k] of a cm-channel pixel):
// the op kind is switched on once per op and group instead of once per
// value.  Same arithmetic as mp_pw_chan; lists longer than three ops are
// read from L.
struct PwRegs {
    int n;
    int op[3];
    float p0[3], p1[3], p2[3];
};

__device__ __forceinline__ PwRegs mp_pw_regs(const PwList &L)
{
    PwRegs r;
    r.n = L.n;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        r.op[i] = L.op[i].op;
        r.p0[i] = L.op[i].p0;
        r.p1[i] = L.op[i].p1;
        r.p2[i] = L.op[i].p2;
    }
    return r;
}

template <int N>
__device__ __forceinline__ void mp_pw_chan_n(const PwRegs &f, const PwList &L, float (&v)[N], const int (&ch)[N],
                                             int cm)
{
    if (f.n > 3) {
        for (int i = 0; i < L.n; ++i)
#pragma unroll
            for (int k = 0; k < N; ++k) v[k] = mp_pw_chan(L.op[i].op, L.op[i].p0, L.op[i].p1, L.op[i].p2, v[k], ch[k], cm);
        return;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (i >= f.n) break;
        const float p0 = f.p0[i], p1 = f.p1[i], p2 = f.p2[i];
        switch (f.op[i]) {
        case MP_OP_BRIGHTNESS:
#pragma unroll
            for (int k = 0; k < N; ++k) v[k] = (cm == 4 && ch[k] == 3) ? v[k] : mp_clamp01(v[k] + p0);
            break;
        case MP_OP_ADJUST_GAMMA:
#pragma unroll
            for (int k = 0; k < N; ++k) v[k] = (cm == 4 && ch[k] == 3) ? v[k] : mp_clamp01(p1 * __powf(v[k], p0));
            break;
        case MP_OP_COLORIZE:
#pragma unroll
            for (int k = 0; k < N; ++k)
                if (cm >= 3 && ch[k] < 3) v[k] = fminf(1.0f, v[k] * (ch[k] == 0 ? p0 : (ch[k] == 1 ? p1 : p2)));
            break;
        default:
            break;
        }
    }
}

// ---------------------------------------------------------------------------
// mbarrier / TMA wrappers (PTX ISA 8.x, sm_90+; compiled for sm_103a).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t mp_smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mp_mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mp_smem_addr(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mp_fence_barrier_init()
{
    // Make the initialised barrier visible to the async (TMA) proxy.
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mp_mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
                     mp_smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mp_mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(mp_smem_addr(bar)) : "memory");
}

// Arrive once `dep` is computed: a thread whose loaded values end in a
// register sum (no store) makes its arrive depend on the sum, so the loads
// have completed before the buffer can be refilled.
__device__ __forceinline__ void mp_mbar_arrive_after(uint64_t *bar, float dep)
{
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(mp_smem_addr(bar)), "f"(dep)
                 : "memory");
}

__device__ __forceinline__ bool mp_mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(mp_smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: returns false if the phase did not complete within `limit`
// polls (MP_SPIN_LIMIT: about two seconds), so a lost transfer turns into an
// error status instead of a hung GPU.
__device__ __forceinline__ bool mp_mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                     uint32_t limit = MP_SPIN_LIMIT)
{
    for (uint32_t i = 0; i < limit; ++i) {
        if (mp_mbar_try_wait(bar, parity)) return true;
        if (i >= MP_SPIN_FAST) __nanosleep(1000);
    }
    return false;
}

__device__ __forceinline__ void mp_tensormap_acquire(const CUtensorMap *map)
{
    // The map may live in global memory (batch job table); order the generic
    // writes that produced it before the TMA unit reads it.
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map) : "memory");
}

__device__ __forceinline__ void mp_tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar,
                                               int x, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%3, %4}], [%2];" ::"r"(mp_smem_addr(dst)),
        "l"(map), "r"(mp_smem_addr(bar)), "r"(x), "r"(y)
        : "memory");
}

// ---------------------------------------------------------------------------
// Host-side helpers shared by the .cu files of the library.
// ---------------------------------------------------------------------------
#ifdef __cplusplus
void mp_set_cuda_error(cudaError_t e);
// Converts a CUDA error into an MPStatus, remembering its text.
MPStatus mp_cuda_status(cudaError_t e);
#define MP_CUDA_TRY(expr)                                    \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) return mp_cuda_status(_e);    \
    } while (0)

// Per-device error word the kernels write (MP_KERR_*).
int *mp_device_error_word(int device);
// Reads and clears the error word; MP_ERROR_KERNEL_TIMEOUT if set.
MPStatus mp_check_device_error(cudaStream_t stream);

// Tensor-map encoder from the driver (looked up at run time).
typedef CUresult (*mp_encode_tiled_fn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                       const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                       const cuuint32_t *, CUtensorMapInterleave,
                                       CUtensorMapSwizzle, CUtensorMapL2promotion,
                                       CUtensorMapFloatOOBfill);
mp_encode_tiled_fn mp_get_encode_tiled();

// Stream-ordered allocation from the device's memory pool.
MPStatus mp_malloc_async(void **p, size_t bytes, cudaStream_t s);
void mp_free_async(void *p, cudaStream_t s);
// Host-to-device copy of a host table that the caller may reuse as soon as
// this returns (staged through a page-locked ring: no wait for the stream).
MPStatus mp_upload_async(void *dst, const void *src, size_t bytes, cudaStream_t s);

// Kernel launchers (mp_kernels.cu).  `jobs` is a device table of njobs jobs
// sorted by tile0; `total_tiles` the sum of their ntiles.
// `tile_job[t]` is the job index of global tile t; `variant` selects the
// channel specialisation (mp_variant) of GAUSS / ROTATE launches.
// `gauss` = {tw, th, rmax, use_tma} for GAUSS launches (persistent grid).
MPStatus mp_launch_kind(int kind, int variant, const MPJob *jobs_dev, const int *tile_job,
                        int total_tiles, size_t smem_bytes, int *err, cudaStream_t s,
                        const int *gauss = nullptr);
// Sets the dynamic shared-memory limit a launch needs; call outside capture.
MPStatus mp_prepare_kind(int kind, int variant, size_t smem_bytes);
// Channel variant of a (source channels, channels after prologue) pair, -1 if none.
int mp_variant(int cin, int cmid);
// Single-job launch with the job passed by value (no device table).
MPStatus mp_launch_single(int kind, const MPJob &job, size_t smem_bytes, cudaStream_t s);
// Adjoint kernels (mp_grad.cu), one job per image, tiles as the forward kinds.
enum { MPK_POINT_ADJ = 10, MPK_ROTATE_ADJ = 11 };
MPStatus mp_launch_adjoint(int kind, const MPJob *jobs_dev, const int *tile_job, int total_tiles,
                           int *err, cudaStream_t s);
// Single-job launch with an explicit device error word (no allocation).
MPStatus mp_launch_single_err(int kind, const MPJob &job, size_t smem_bytes, int *err, cudaStream_t s);
// Runs the stages on one image, intermediates in the two caller-provided
// device buffers of half_bytes each; allocates no device memory.  With
// launch = false it only validates (descriptors, parameters, intermediate
// sizes) and launches nothing.
MPStatus mp_run_image_noalloc(const MPStage *stages, int nstages, uint64_t seed, uint64_t index,
                              const MPImage &in, const MPImage &out, void *half0, void *half1,
                              size_t half_bytes, int *err, cudaStream_t s, bool launch);
// The reference's own layouts (uint8 RGBA / uint8 RGB for rgb2grey /
// float64 greyscale) and arithmetic, in place on an object (mp_legacy.cu).
MPStatus mp_legacy_apply(MPObjData *o, int op, double p0, double p1, double p2);
// In-place channel-agnostic pointwise list over n contiguous floats.
MPStatus mp_launch_flat(float *data, size_t n, const PwList &L, cudaStream_t s);
// Dynamic shared memory a GAUSS launch needs for the given geometry.
size_t mp_gauss_smem_bytes(int tw, int th, int radius, int cin, int cmid, int has_pro);
// Footprint-staged rotate (mp_rot.cu): `buf_floats` = floats of one
// footprint buffer (the largest box of the launch, 128-byte multiple).
MPStatus mp_ro_prepare(int c, size_t smem, int *ctas_per_sm);
MPStatus mp_ro_launch(int c, const MPJob *jobs_dev, const int *tile_job, int total, int buf_floats, int grid,
                      int *err, cudaStream_t s);
MPStatus mp_ro_launch_single(int c, const MPJob &job, int buf_floats, int grid, int *err, cudaStream_t s);
size_t mp_ro_smem(int buf_floats);
// Streaming gaussian of mp_vh.cuh (mp_vh*.cu, mp_vc*.cu, mp_vb*.cu).  A
// kernel code names the family: the source channel count (1, 3, 4) for the
// single-channel family (cmid 1), 4 + C (7, 8) for the channel-preserving
// family on C = 3 or 4 interleaved channels, plus 16 for the radius buckets
// above MP_VH_RMAX (1-channel sources, RGB and RGBA only), plus 32 for the
// dot mode of the gaussian's adjoint (mp_vd*.cu), plus 64 / 128 for the RGB
// channel-preserving kernels of radii 1..4 / 5..8 (mp_vc_c3_lo.cu,
// mp_vc_c3_mid.cu: own register budgets, 4 CTAs per SM); -1 if no kernel
// takes (cin, cmid, radius).  mp_vh_bucket is the radius a job runs with
// (its strip halo).  Strips are counted in columns: pixels when cm = 1,
// floats of the interleaved row otherwise.
int mp_vh_code(int cin, int cmid, int radius);
int mp_vh_bucket(int radius);
// Code of the d sigma dot mode (code + 32) for c-channel images, radii up
// to MP_VH_RMAX; -1 if none.
int mp_vh_dot_code(int c, int radius);
int mp_vh_strip(int radius, int cm);
int mp_vh_fit_strip(int radius, int w, int cm);
// Tuned cap on strip widths (columns, a multiple of 8 from 64; 0: none).
void mp_vh_set_strip_cap(int cols);
MPStatus mp_vh_prepare(int code, int *ctas_per_sm);
MPStatus mp_vh_launch(int code, const MPJob *jobs_dev, const int *tile_job, int total, int grid, int *err,
                      int *counter, cudaStream_t s);
MPStatus mp_vh_launch_single(int code, const MPJob &job, int grid, int *err, cudaStream_t s);

// Fused gaussian -> rotate (mp_fuse.cu): one output tile is 64 x 64 pixels
// of the one-channel result.  mp_fz_geom sizes the shared memory for the
// largest footprint box (pixels), radius and source channel count of a
// launch; mp_fz_prepare raises the kernel's shared-memory limit and returns
// the resident CTAs per SM (call outside capture).
#define MP_FZ_RMAX 12
#define MP_FZ_CR 16    // source rows per TMA chunk (the tensor map's box height)
bool mp_fz_supported(int cin, int radius);
FzGeom mp_fz_geom(int box_max, int rmax, int cin, size_t *smem);
MPStatus mp_fz_prepare(int cin, size_t smem, int *ctas_per_sm);
MPStatus mp_fz_launch(int cin, const MPJob *jobs_dev, const int *tile_job, int total, const FzGeom &g, size_t smem,
                      int grid, int *err, cudaStream_t s);

// Streaming gaussian (mp_stream.cu).  mp_gs_prepare raises the
// shared-memory limit and returns the resident CTAs per SM (call outside
// capture); mp_gs_launch runs `grid` persistent CTAs over `total` strip
// items of a job table.
MPStatus mp_gs_prepare(int variant, size_t smem, int *ctas_per_sm);
MPStatus mp_gs_launch(int variant, const MPJob *jobs_dev, const int *tile_job, int total, const GsGeom &g,
                      int grid, int *err, cudaStream_t s);
MPStatus mp_gs_launch_single(int variant, const MPJob &job, const GsGeom &g, int grid, int *err,
                             cudaStream_t s);
#endif
