// mp_legacy.cu -- the reference's own layouts and arithmetic, on sm_103a.
//
// The reference's kernels (src/millipyde_image.cpp:50-524) work on packed
// uint8 RGBA pixels and float64 greyscale; their results define what its
// Python tests check.  This file reproduces them so objects in those layouts
// (e.g. PNGs loaded as uint8 RGBA) behave as under the reference:
//   rgb2grey   uint8 (3 or 4 channels) -> float64 fmin(1, (0.2125r+0.7154g+0.0721b)/255)
//   transpose, fliplr   any pixel of 4 (RGBA) or 8 (float64) bytes, exact
//   rotate     nearest pixel by truncation toward zero, zero outside
//   gaussian   radius 8, weights expf(-k^2/2s^2) normalised on the host;
//              float64: row then column pass, fmax(0, .), no FMA contraction
//              (the reference's sum += a*b order); RGBA: per byte lane, every
//              tap product truncated to int, lane sums mod 256, the column
//              pass forcing byte 3 to 0xff
//   brightness / adjust_gamma / colorize
//              float64: clamp01(x + d), clamp01(gain * powf(x, g));
//              RGBA: 256-entry tables per colour channel built on the host with
//              the reference's formulas (char delta, powf, truncation), alpha kept
// The tables and tap products make the byte results bit-identical to the
// reference's arithmetic (tests/golden/reference_ops.npz).
#include <math.h>
#include <string.h>

#include "mp_internal.cuh"

#define LG_R 8
#define LG_TAPS (2 * LG_R + 1)

struct LgJob {
    const unsigned char *src;
    unsigned char *dst;
    int h, w;                // source geometry
    int ho, wo;              // output geometry
    int sp, dp;              // pitches in bytes
    int cin;                 // source channels (uint8 grey conversion)
    int psize;               // pixel bytes for permutations (4 or 8)
    double c, s;             // rotate cos / sin
    double wts[LG_TAPS];     // gaussian taps (float64 path)
    int tap_tbl[LG_TAPS][256];   // gaussian RGBA: (int)(b * w[i])
    unsigned char lut[3][256];   // RGBA pointwise tables
    double p0, p1;           // float64 pointwise parameters
};

// ---------------------------------------------------------------- kernels
__global__ void lg_grey_u8(const __grid_constant__ LgJob J)
{
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= J.w || y >= J.h) return;
    const unsigned char *p = J.src + (size_t)y * J.sp + (size_t)x * J.cin;
    const double r = p[0], g = p[1], b = p[2];
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(0.2125, r), __dmul_rn(0.7154, g)), __dmul_rn(0.0721, b));
    reinterpret_cast<double *>(J.dst + (size_t)y * J.dp)[x] = fmin(1.0, s / 255);
}

template <typename T>
__global__ void lg_permute(const __grid_constant__ LgJob J, int transpose)
{
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= J.w || y >= J.h) return;
    const T v = reinterpret_cast<const T *>(J.src + (size_t)y * J.sp)[x];
    if (transpose) reinterpret_cast<T *>(J.dst + (size_t)x * J.dp)[y] = v;
    else reinterpret_cast<T *>(J.dst + (size_t)y * J.dp)[J.w - 1 - x] = v;
}

template <typename T>
__global__ void lg_rotate(const __grid_constant__ LgJob J)
{
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= J.w || y >= J.h) return;
    const double hw = (double)J.w / 2, hh = (double)J.h / 2;
    const double dx = (double)x - hw, dy = (double)y - hh;
    // same operation order as the reference's host-free expression, no FMA
    const int xr = (int)__dadd_rn(__dsub_rn(__dmul_rn(dx, J.c), __dmul_rn(dy, J.s)), hw);
    const int yr = (int)__dadd_rn(__dadd_rn(__dmul_rn(dx, J.s), __dmul_rn(dy, J.c)), hh);
    T v = (T)0;
    if (xr >= 0 && xr < J.w && yr >= 0 && yr < J.h) v = reinterpret_cast<const T *>(J.src + (size_t)yr * J.sp)[xr];
    reinterpret_cast<T *>(J.dst + (size_t)y * J.dp)[x] = v;
}

__global__ void lg_gauss_f64(const __grid_constant__ LgJob J, int pass, const double *tmp_in, double *tmp_out)
{
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= J.w || y >= J.h) return;
    double sum = 0.0;
    if (pass == 0) {   // row pass: source -> tmp
        const double *row = reinterpret_cast<const double *>(J.src + (size_t)y * J.sp);
        for (int k = -LG_R; k <= LG_R; ++k) {
            const int xx = x + k;
            const double v = (xx >= 0 && xx < J.w) ? row[xx] : 0.0;
            sum = __dadd_rn(sum, __dmul_rn(v, J.wts[LG_R - k]));
        }
        tmp_out[(size_t)y * J.w + x] = sum;
    } else {           // column pass: tmp -> destination, fmax(0, .)
        for (int k = -LG_R; k <= LG_R; ++k) {
            const int yy = y + k;
            const double v = (yy >= 0 && yy < J.h) ? tmp_in[(size_t)yy * J.w + x] : 0.0;
            sum = __dadd_rn(sum, __dmul_rn(v, J.wts[LG_R - k]));
        }
        reinterpret_cast<double *>(J.dst + (size_t)y * J.dp)[x] = fmax(0.0, sum);
    }
}

__global__ void lg_gauss_rgba(const __grid_constant__ LgJob J, int pass, const unsigned int *tmp_in,
                              unsigned int *tmp_out)
{
    __shared__ int tbl[LG_TAPS][256];
    for (int i = threadIdx.y * 32 + threadIdx.x; i < LG_TAPS * 256; i += 256)
        tbl[i >> 8][i & 255] = J.tap_tbl[i >> 8][i & 255];
    __syncthreads();
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= J.w || y >= J.h) return;
    int s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    for (int k = -LG_R; k <= LG_R; ++k) {
        unsigned int px = 0;
        if (pass == 0) {
            const int xx = x + k;
            if (xx >= 0 && xx < J.w) px = reinterpret_cast<const unsigned int *>(J.src + (size_t)y * J.sp)[xx];
        } else {
            const int yy = y + k;
            if (yy >= 0 && yy < J.h) px = tmp_in[(size_t)yy * J.w + x];
        }
        const int *t = tbl[LG_R - k];
        s0 += t[px & 0xff];
        s1 += t[(px >> 8) & 0xff];
        s2 += t[(px >> 16) & 0xff];
        s3 += t[(px >> 24) & 0xff];
    }
    if (pass == 0) {
        tmp_out[(size_t)y * J.w + x] = (unsigned)(s0 & 0xff) | ((unsigned)(s1 & 0xff) << 8) |
                                       ((unsigned)(s2 & 0xff) << 16) | ((unsigned)(s3 & 0xff) << 24);
    } else {
        reinterpret_cast<unsigned int *>(J.dst + (size_t)y * J.dp)[x] =
            (unsigned)(s0 & 0xff) | ((unsigned)(s1 & 0xff) << 8) | ((unsigned)(s2 & 0xff) << 16) | 0xff000000u;
    }
}

// op: 0 brightness, 1 gamma (float64 path); RGBA path uses the tables
__global__ void lg_point(const __grid_constant__ LgJob J, int rgba, int op)
{
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= J.w || y >= J.h) return;
    if (rgba) {
        const unsigned char *p = J.src + (size_t)y * J.sp + (size_t)x * 4;
        unsigned char *d = J.dst + (size_t)y * J.dp + (size_t)x * 4;
        d[0] = J.lut[0][p[0]];
        d[1] = J.lut[1][p[1]];
        d[2] = J.lut[2][p[2]];
        d[3] = p[3];
    } else {
        const double v = reinterpret_cast<const double *>(J.src + (size_t)y * J.sp)[x];
        double r;
        if (op == 0) {
            r = v + J.p0;
        } else {
            r = J.p1 * (double)powf((float)v, (float)J.p0);
        }
        r = r < 0 ? 0 : r;
        r = r > 1 ? 1 : r;
        reinterpret_cast<double *>(J.dst + (size_t)y * J.dp)[x] = r;
    }
}

// ---------------------------------------------------------------- host side
#define NPY_UBYTE_T 2
#define NPY_DOUBLE_T 12

static int lg_round16(long long v) { return (int)((v + 15) / 16 * 16); }

// Which legacy layout an object is: 1 uint8 RGBA, 2 uint8 RGB, 3 float64 grey, 0 none.
static int lg_layout(const MPObjData *o)
{
    if (o->type == NPY_UBYTE_T && o->ndims == 3 && o->dims[2] == 4) return 1;
    if (o->type == NPY_UBYTE_T && o->ndims == 3 && o->dims[2] == 3) return 2;
    if (o->type == NPY_DOUBLE_T && o->ndims == 2) return 3;
    return 0;
}

static MPStatus lg_set(MPObjData *o, void *data, int h, int w, int c, int itemsize, int type, int pitch)
{
    const int nd = (c == 1) ? 2 : 3;
    int *dims = (int *)malloc(sizeof(int) * 2 * nd);
    if (!dims) return MP_ERROR_OUT_OF_MEMORY;
    dims[0] = h;
    dims[1] = w;
    if (nd == 3) dims[2] = c;
    dims[nd] = pitch;
    dims[nd + 1] = (nd == 3) ? c * itemsize : itemsize;
    if (nd == 3) dims[nd + 2] = itemsize;
    if (o->device_data && o->device_data != data) mp_free_async(o->device_data, (cudaStream_t)o->stream);
    free(o->dims);
    o->dims = dims;
    o->ndims = nd;
    o->device_data = data;
    o->type = type;
    o->nbytes = (size_t)h * pitch;
    return MILLIPYDE_SUCCESS;
}

static void lg_char_lut(unsigned char lut[256], double delta)
{
    // char(delta * 255): truncation toward zero, two's-complement wrap
    int d = (int)trunc(delta * 255) & 0xff;
    if (d >= 128) d -= 256;
    for (int b = 0; b < 256; ++b) {
        int v = b + d;
        if (d > 0) v = v > 255 ? 255 : v;
        else v = v < 0 ? 0 : v;
        lut[b] = (unsigned char)v;
    }
}

// Runs a legacy op on an object: MP_ERROR_UNSUPPORTED_TYPE if the object is
// not in a layout the reference handled for this op.
MPStatus mp_legacy_apply(MPObjData *o, int op, double p0, double p1, double p2)
{
    const int lay = lg_layout(o);
    if (!lay) return MP_ERROR_UNSUPPORTED_TYPE;
    if (lay == 2 && op != MP_OP_RGB2GREY) return MP_ERROR_UNSUPPORTED_TYPE;
    if (lay == 3 && op == MP_OP_RGB2GREY) return MILLIPYDE_SUCCESS;   // already grey
    if (lay == 3 && op == MP_OP_COLORIZE) return MILLIPYDE_SUCCESS;   // no colour to scale
    const int h = o->dims[0], w = o->dims[1];
    if ((long long)h * w == 0) return MILLIPYDE_SUCCESS;
    if (!o->device_data) return MP_ERROR_NULL_DATA;
    MP_CUDA_TRY(cudaSetDevice(o->mem_loc));
    cudaStream_t s = (cudaStream_t)o->stream;
    LgJob *J = (LgJob *)calloc(1, sizeof(LgJob));
    if (!J) return MP_ERROR_OUT_OF_MEMORY;
    J->src = (const unsigned char *)o->device_data;
    J->h = h;
    J->w = w;
    J->sp = o->dims[o->ndims];
    J->cin = lay == 3 ? 1 : o->dims[2];
    J->psize = lay == 3 ? 8 : 4;
    const dim3 blk(32, 8), grd((w + 31) / 32, (h + 7) / 8);
    MPStatus st = MILLIPYDE_SUCCESS;
    void *out = nullptr, *tmp = nullptr;
    int oh = h, ow = w, oc = lay == 3 ? 1 : 4, oitem = lay == 3 ? 8 : 1, otype = o->type;
    switch (op) {
    case MP_OP_RGB2GREY:
        oc = 1;
        oitem = 8;
        otype = NPY_DOUBLE_T;
        break;
    case MP_OP_TRANSPOSE:
        oh = w;
        ow = h;
        break;
    case MP_OP_GAUSSIAN:
        if (!(p0 > 0.0) || !isfinite(p0)) { free(J); return MP_ERROR_INVALID_ARGS; }
        break;
    case MP_OP_ROTATE:
        if (!isfinite(p0)) { free(J); return MP_ERROR_INVALID_ARGS; }
        break;
    default:
        break;
    }
    const int opitch = lg_round16((long long)ow * oc * oitem);
    J->ho = oh;
    J->wo = ow;
    J->dp = opitch;
    st = mp_malloc_async(&out, (size_t)oh * opitch, s);
    if (st != MILLIPYDE_SUCCESS) { free(J); return st; }
    J->dst = (unsigned char *)out;
    cudaError_t e = cudaSuccess;
    switch (op) {
    case MP_OP_RGB2GREY:
        lg_grey_u8<<<grd, blk, 0, s>>>(*J);
        break;
    case MP_OP_TRANSPOSE:
    case MP_OP_FLIPLR:
        if (lay == 3) lg_permute<unsigned long long><<<grd, blk, 0, s>>>(*J, op == MP_OP_TRANSPOSE);
        else lg_permute<unsigned int><<<grd, blk, 0, s>>>(*J, op == MP_OP_TRANSPOSE);
        break;
    case MP_OP_ROTATE: {
        const double a = p0 * 0.01745329252;   // src/millipyde_image.cpp:702
        J->c = cos(a);
        J->s = sin(a);
        if (lay == 3) lg_rotate<unsigned long long><<<grd, blk, 0, s>>>(*J);
        else lg_rotate<unsigned int><<<grd, blk, 0, s>>>(*J);
        break;
    }
    case MP_OP_GAUSSIAN: {
        double e0[LG_TAPS], sum = 0;
        for (int i = 0; i < LG_TAPS; ++i) {
            const int dist = -1 * (LG_R - i);
            e0[i] = (double)expf((float)(-1 * ((dist * dist) / (2 * p0 * p0))));
            sum += e0[i];
        }
        for (int i = 0; i < LG_TAPS; ++i) J->wts[i] = e0[i] / sum;
        for (int i = 0; i < LG_TAPS; ++i)
            for (int b = 0; b < 256; ++b) J->tap_tbl[i][b] = (int)((double)b * J->wts[i]);
        st = mp_malloc_async(&tmp, (size_t)h * w * (lay == 3 ? 8 : 4), s);
        if (st != MILLIPYDE_SUCCESS) break;
        if (lay == 3) {
            lg_gauss_f64<<<grd, blk, 0, s>>>(*J, 0, nullptr, (double *)tmp);
            lg_gauss_f64<<<grd, blk, 0, s>>>(*J, 1, (const double *)tmp, nullptr);
        } else {
            lg_gauss_rgba<<<grd, blk, 0, s>>>(*J, 0, nullptr, (unsigned int *)tmp);
            lg_gauss_rgba<<<grd, blk, 0, s>>>(*J, 1, (const unsigned int *)tmp, nullptr);
        }
        break;
    }
    case MP_OP_BRIGHTNESS:
        if (lay == 3) {
            J->p0 = p0;
            lg_point<<<grd, blk, 0, s>>>(*J, 0, 0);
        } else {
            for (int c = 0; c < 3; ++c) lg_char_lut(J->lut[c], p0);
            lg_point<<<grd, blk, 0, s>>>(*J, 1, 0);
        }
        break;
    case MP_OP_ADJUST_GAMMA:
        if (lay == 3) {
            J->p0 = p0;
            J->p1 = p1;
            lg_point<<<grd, blk, 0, s>>>(*J, 0, 1);
        } else {
            for (int b = 0; b < 256; ++b) {
                double t = p1 * (255 * (double)powf((float)((double)b / 255), (float)p0));
                t = t < 0 ? 0 : t;
                const unsigned char v = t > 255 ? 255 : (unsigned char)t;
                J->lut[0][b] = J->lut[1][b] = J->lut[2][b] = v;
            }
            lg_point<<<grd, blk, 0, s>>>(*J, 1, 1);
        }
        break;
    case MP_OP_COLORIZE: {
        const double m[3] = {p0, p1, p2};
        for (int c = 0; c < 3; ++c)
            for (int b = 0; b < 256; ++b) {
                const double t = (double)b * m[c];
                J->lut[c][b] = t > 255 ? 255 : (unsigned char)t;
            }
        lg_point<<<grd, blk, 0, s>>>(*J, 1, 2);
        break;
    }
    default:
        st = MP_ERROR_BAD_DESCRIPTOR;
    }
    if (st == MILLIPYDE_SUCCESS) {
        e = cudaGetLastError();
        if (e != cudaSuccess) st = mp_cuda_status(e);
    }
    mp_free_async(tmp, s);
    free(J);
    if (st != MILLIPYDE_SUCCESS) {
        mp_free_async(out, s);
        return st;
    }
    return lg_set(o, out, oh, ow, oc, oitem, otype, opitch);
}
