// mp_kernels.cu -- sm_103a kernels of the image hot path.
//
// Four segment kernels, each able to run a pointwise prologue (applied to
// every source value it reads) and a pointwise epilogue (applied to every
// value it writes), plus an optional fliplr output map:
//   POINT      pointwise only                       (rgb2grey, brightness, gamma, colorize, fliplr)
//   GAUSS      separable zero-padded gaussian       (src/millipyde_image.cpp:146-244, radius ceil(3 sigma))
//   ROTATE     bilinear rotation about (W/2, H/2)   (src/millipyde_image.cpp:114-139 geometry)
//   TRANSPOSE  out[x][y] = in[y][x]                 (src/millipyde_image.cpp:73-96)
// Every kernel reads its work from an MPJob (one per image).  A launch covers
// a ragged batch: blockIdx.x is a global tile index, mapped to its image by a
// per-tile job index built with the plan.  GAUSS and ROTATE are compiled per
// channel variant (source channels, channels after the prologue).
#include <algorithm>
#include <mutex>
#include <utility>
#include <vector>

#include "mp_internal.cuh"

#define MP_THREADS 256

// ---------------------------------------------------------------------------
// GAUSS shared-memory layout (host and device agree on it).
//   [0,16)        mbarrier
//   [16, ...)     vertical taps, horizontal taps (MP_MAX_TAPS rounded to 16
//                 floats each), 32 floats of reduction scratch
//   A (128-B aligned): TMA tile S, later vT (prologue) or obuf (no prologue)
//   B (128-B aligned): vT (no prologue) or G then obuf (prologue)
// All sizes in floats unless noted.
// ---------------------------------------------------------------------------
struct GaussGeom {
    int BH, nbx_max, JW, GWp, RBp, OBW;
    int offA, offB;      // byte offsets from the 128-B aligned base
    int total;           // bytes
};

__host__ __device__ __forceinline__ int mp_round_up(int a, int b) { return (a + b - 1) / b * b; }

__host__ __device__ __forceinline__ GaussGeom mp_gauss_geom(int tw, int th, int r, int cin,
                                                            int cmid, int has_pro)
{
    GaussGeom g;
    g.BH = th + 2 * r;
    g.nbx_max = (3 + (tw + 2 * r) * cin + 63) / 64;
    g.JW = (tw + 2 * r) * cmid;
    g.GWp = mp_round_up(g.JW, 4);
    g.RBp = th + 4;
    g.OBW = tw * cmid + 1;
    const int S = g.nbx_max * 64 * g.BH;
    const int vT = g.JW * g.RBp;
    const int G = has_pro ? g.BH * g.GWp : 0;
    const int ob = th * g.OBW;
    int A, B;
    if (has_pro) {
        A = S > vT ? S : vT;
        B = G > ob ? G : ob;
    } else {
        A = S > ob ? S : ob;
        B = vT;
    }
    const int head = mp_round_up(16 + 8 * mp_round_up(MP_MAX_TAPS, 16) + 4 * 32, 128);
    g.offA = head;
    g.offB = g.offA + mp_round_up(A * 4, 128);
    g.total = g.offB + mp_round_up(B * 4, 128);
    return g;
}

size_t mp_gauss_smem_bytes(int tw, int th, int radius, int cin, int cmid, int has_pro)
{
    return (size_t)mp_gauss_geom(tw, th, radius, cin, cmid, has_pro).total + 128;  // +128: alignment slack
}

// Block-wide sum of one float per thread, added (FP64) to *acc by thread 0.
// `red` is 32 floats of shared memory.  All threads of the block must call.
__device__ __forceinline__ void mp_block_add(float v, float *red, double *acc)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        atomicAdd(acc, (double)t);
    }
}

// 1-D correlation along the row index of a [rows][stride] float array,
// producing 8 consecutive outputs for 4 consecutive columns:
//   acc[o] += sum_{m<ntaps} w[m] * base[(o+m)*stride .. +3]
// Inputs are kept in an 8-entry register ring indexed by row & 7, so each
// loaded float4 feeds 8 outputs (8 FMAs per float loaded).
__device__ __forceinline__ void mp_conv8(const float *base, int stride, int ntaps,
                                         const float *w, float4 acc[8])
{
    float4 X[8];
#pragma unroll
    for (int k = 0; k < 7; ++k) X[k] = *reinterpret_cast<const float4 *>(base + k * stride);
    for (int m0 = 0; m0 < ntaps; m0 += 8) {
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const int m = m0 + s;
            if (m >= ntaps) break;
            X[(s + 7) & 7] = *reinterpret_cast<const float4 *>(base + (m + 7) * stride);
            const float wm = w[m];
#pragma unroll
            for (int o = 0; o < 8; ++o) {
                const float4 x = X[(s + o) & 7];
                acc[o].x = fmaf(wm, x.x, acc[o].x);
                acc[o].y = fmaf(wm, x.y, acc[o].y);
                acc[o].z = fmaf(wm, x.z, acc[o].z);
                acc[o].w = fmaf(wm, x.w, acc[o].w);
            }
        }
    }
}

// Channel-count variants the GAUSS and ROTATE kernels are compiled for:
// (source channels, channels after the prologue).
template <int V> struct MPChan;
template <> struct MPChan<0> { static constexpr int CIN = 1, CMID = 1; };
template <> struct MPChan<1> { static constexpr int CIN = 3, CMID = 3; };
template <> struct MPChan<2> { static constexpr int CIN = 4, CMID = 4; };
template <> struct MPChan<3> { static constexpr int CIN = 3, CMID = 1; };
template <> struct MPChan<4> { static constexpr int CIN = 4, CMID = 1; };

// One output tile (tw x th pixels) of a separable gaussian.
//   1. TMA loads the halo'd source tile (th+2r rows, (tw+2r)*cin floats plus
//      up to 3 floats of 16-byte alignment slack) as nbx boxes of 64 floats;
//      rows/columns outside the image arrive as zeros (the zero padding).
//   2. Optional prologue: pointwise ops into G (zeros kept outside the image).
//   3. Vertical pass -> vT, stored transposed ([column][row]).
//   4. Horizontal pass over vT rows -> obuf ([row][x*cmid+c]).
//   5. Copy-out with epilogue and the fliplr map (or, in dot mode, the sum of
//      out * aux over the tile).
// Loops over 2-D index ranges run warp-per-row / lane-per-column, so no
// integer division sits in a per-element loop.
template <int CIN, int CMID>
__device__ __forceinline__ void mp_gauss_tile(const MPJob &J, int t, unsigned char *smem_raw,
                                              bool map_in_global, int *err)
{
    const int r = J.radius, tw = J.tw, th = J.th;
    const int H = J.h, W = J.w;
    const int ty = t / J.tiles_x, tx = t - ty * J.tiles_x;
    const int x0 = tx * tw, y0 = ty * th;
    const int has_pro = J.pro.n > 0;
    const GaussGeom g = mp_gauss_geom(tw, th, r, CIN, CMID, has_pro);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;

    unsigned char *base =
        smem_raw + ((128 - (int)(mp_smem_addr(smem_raw) & 127)) & 127);
    uint64_t *bar = reinterpret_cast<uint64_t *>(base);
    float *wsm = reinterpret_cast<float *>(base + 16);
    float *wsm_h = wsm + mp_round_up(MP_MAX_TAPS, 16);
    float *red = wsm_h + mp_round_up(MP_MAX_TAPS, 16);
    float *A = reinterpret_cast<float *>(base + g.offA);
    float *B = reinterpret_cast<float *>(base + g.offB);
    float *S = A;

    const int gx = (x0 - r) * CIN;
    const int xa = gx & ~3;
    const int delta = gx - xa;
    const int nbx = (delta + (tw + 2 * r) * CIN + 63) / 64;
    const int ntaps = 2 * r + 1;
    const int boxs = 64 * g.BH;           // floats per TMA box

    for (int i = threadIdx.x; i < ntaps; i += blockDim.x) {
        wsm[i] = J.wts[i];
        wsm_h[i] = J.hsep ? J.wts_h[i] : J.wts[i];
    }

    if (J.use_tma) {
        if (threadIdx.x == 0) {
            mp_mbar_init(bar, 1);
            mp_fence_barrier_init();
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            if (map_in_global) mp_tensormap_acquire(&J.tmap);
            mp_mbar_arrive_expect_tx(bar, (uint32_t)(nbx * boxs * 4));
            for (int b = 0; b < nbx; ++b)
                mp_tma_load_2d(S + b * boxs, &J.tmap, bar, xa + 64 * b, y0 - r);
        }
        const bool ok = mp_mbar_wait_bounded(bar, 0);
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0) atomicExch(err, MP_KERR_TIMEOUT);
            mp_mbar_wait_bounded(bar, 0);   // let in-flight copies land before exiting
            return;
        }
    } else {
        // Plain-load fallback for sources whose rows are not 16-byte aligned:
        // same box-major layout, zeros outside the image.
        const int rowlen = W * CIN;
        const float *src = J.src;
        const int sp = J.src_pitch;
        for (int b = 0; b < nbx; ++b) {
            for (int row = warp; row < g.BH; row += nwarps) {
                const int gyy = y0 - r + row;
                const bool rowin = gyy >= 0 && gyy < H;
                for (int col = lane; col < 64; col += 32) {
                    const int gxx = xa + 64 * b + col;
                    float v = 0.0f;
                    if (rowin && gxx >= 0 && gxx < rowlen) v = __ldg(src + (size_t)gyy * sp + gxx);
                    S[b * boxs + row * 64 + col] = v;
                }
            }
        }
        __syncthreads();
    }

    // ---- 2. prologue into G
    const float *vsrc;
    int vstride, vdelta, nq;
    float *vT;
    float *obuf;
    if (has_pro) {
        float *G = B;
        const int npx = tw + 2 * r;
        const PwFast pro = mp_pw_fast(J.pro);
        for (int row = warp; row < g.BH; row += nwarps) {
            const int gyy = y0 - r + row;
            const bool rowin = gyy >= 0 && gyy < H;
            const float *Srow = S + row * 64;
            float *Grow = G + row * g.GWp;
            for (int xi = lane; xi < npx; xi += 32) {
                const int gxx = x0 - r + xi;
                float v[4] = {0.f, 0.f, 0.f, 0.f};
                if (rowin && gxx >= 0 && gxx < W) {
#pragma unroll
                    for (int c = 0; c < CIN; ++c) {
                        const int col = delta + xi * CIN + c;
                        v[c] = Srow[(col >> 6) * boxs + (col & 63)];
                    }
                    mp_pw_apply_f(pro, J.pro, v, CIN);
                }
#pragma unroll
                for (int c = 0; c < CMID; ++c) Grow[xi * CMID + c] = v[c];
            }
        }
        __syncthreads();
        vsrc = G;
        vstride = g.GWp;
        vdelta = 0;
        nq = g.GWp / 4;
        vT = A;
        obuf = B;
    } else {
        vsrc = S;
        vstride = 64;
        vdelta = delta;
        nq = (delta + g.JW + 3) / 4;
        vT = B;
        obuf = A;
    }

    // ---- 3. vertical pass: item (q, grp) = 4 columns x 8 output rows
    const int ngrp = th / 8;
    for (int it = threadIdx.x; it < nq * ngrp; it += blockDim.x) {
        const int grp = it / nq, q = it - grp * nq;
        const float *colbase;
        if (has_pro) colbase = vsrc + 4 * q;
        else colbase = vsrc + (q >> 4) * boxs + ((q & 15) << 2);
        float4 acc[8];
#pragma unroll
        for (int o = 0; o < 8; ++o) acc[o] = make_float4(0.f, 0.f, 0.f, 0.f);
        mp_conv8(colbase + 8 * grp * vstride, vstride, ntaps, wsm, acc);
        const int j0 = 4 * q - vdelta;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int j = j0 + k;
            if (j >= 0 && j < g.JW) {
                float *dst = vT + j * g.RBp + 8 * grp;
                float c0[8];
#pragma unroll
                for (int o = 0; o < 8; ++o)
                    c0[o] = (k == 0) ? acc[o].x : (k == 1) ? acc[o].y : (k == 2) ? acc[o].z : acc[o].w;
                reinterpret_cast<float4 *>(dst)[0] = make_float4(c0[0], c0[1], c0[2], c0[3]);
                reinterpret_cast<float4 *>(dst)[1] = make_float4(c0[4], c0[5], c0[6], c0[7]);
            }
        }
    }
    __syncthreads();

    // ---- 4. horizontal pass: item (a, c, b) = 4 rows x 8 consecutive x, channel c
    const int na = th / 4, nb = tw / 8;
    for (int it = threadIdx.x; it < na * CMID * nb; it += blockDim.x) {
        const int rest = it / na, a = it - rest * na;
        const int b = rest / CMID, c = rest - b * CMID;
        float4 acc[8];
#pragma unroll
        for (int o = 0; o < 8; ++o) acc[o] = make_float4(0.f, 0.f, 0.f, 0.f);
        mp_conv8(vT + ((8 * b) * CMID + c) * g.RBp + 4 * a, CMID * g.RBp, ntaps, wsm_h, acc);
#pragma unroll
        for (int o = 0; o < 8; ++o) {
            float *dst = obuf + (4 * a) * g.OBW + (8 * b + o) * CMID + c;
            dst[0] = acc[o].x;
            dst[g.OBW] = acc[o].y;
            dst[2 * g.OBW] = acc[o].z;
            dst[3 * g.OBW] = acc[o].w;
        }
    }
    __syncthreads();

    // ---- 5a. dot mode: sum(out * aux) over the tile into acc[0]
    if (J.dot) {
        float part = 0.f;
        for (int tt = warp; tt < th; tt += nwarps) {
            const int gyy = y0 + tt;
            if (gyy >= H) break;
            const float *arow = J.aux + (size_t)gyy * J.aux_pitch;
            for (int xx = lane; xx < tw; xx += 32) {
                const int gxx = x0 + xx;
                if (gxx >= W) break;
#pragma unroll
                for (int c = 0; c < CMID; ++c)
                    part = fmaf(obuf[tt * g.OBW + xx * CMID + c], arow[(size_t)gxx * CMID + c], part);
            }
        }
        mp_block_add(part, red, J.acc);
        return;
    }
    // ---- 5. copy-out with epilogue and output map
    const PwFast epi = mp_pw_fast(J.epi);
    const int flip = J.flip, wo = J.wo;
    float *dstb = J.dst;
    const int dp = J.dst_pitch;
    for (int tt = warp; tt < th; tt += nwarps) {
        const int gyy = y0 + tt;
        if (gyy >= H) break;
        float *drow = dstb + (size_t)gyy * dp;
        const float *orow = obuf + tt * g.OBW;
        for (int xx = lane; xx < tw; xx += 32) {
            const int gxx = x0 + xx;
            if (gxx >= W) break;
            float v[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int c = 0; c < CMID; ++c) v[c] = orow[xx * CMID + c];
            const int xo = flip ? (wo - 1 - gxx) : gxx;
            if (epi.n == 0) {
                float *d = drow + (size_t)xo * CMID;
#pragma unroll
                for (int c = 0; c < CMID; ++c) d[c] = v[c];
            } else {
                const int co = mp_pw_apply_f(epi, J.epi, v, CMID);
                float *d = drow + (size_t)xo * co;
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (c < co) d[c] = v[c];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// ROTATE: 32x32 output tile, 256 threads, 4 rows per thread.  Source
// coordinates in 64-bit fixed point (MP_FIX_FRAC fractional bits), so the
// bilinear fractions keep ~24 correct bits even for 8192-wide images; a
// thread steps its coordinates exactly from one of its rows to the next.
//   s = R(theta) (p - c) + c,  c = (W/2, H/2),  p = output pixel
// Neighbours outside the source contribute 0 (zero fill); the prologue is
// applied to each in-range neighbour before interpolation.
// ---------------------------------------------------------------------------
template <int CIN>
__device__ __forceinline__ void mp_load_px(const MPJob &J, int ix, int iy, float v[4])
{
    v[0] = v[1] = v[2] = v[3] = 0.f;
    if (ix < 0 || iy < 0 || ix >= J.w || iy >= J.h) return;
    const float *p = J.src + (size_t)iy * J.src_pitch + (size_t)ix * CIN;
#pragma unroll
    for (int c = 0; c < CIN; ++c) v[c] = __ldg(p + c);
    if (J.pro.n) mp_pw_apply(J.pro, v, CIN);
}

template <int CIN, int CMID>
__device__ __forceinline__ void mp_rotate_tile(const MPJob &J, int t)
{
    const int ty = t / J.tiles_x, tx = t - ty * J.tiles_x;
    const int x = tx * 32 + (threadIdx.x & 31);
    if (x >= J.wo) return;
    const int W = J.w, H = J.h, ho = J.ho;
    const float *src = J.src;
    const int sp = J.src_pitch;
    const long long cosq = J.cosq, sinq = J.sinq;
    const long long X2 = 2LL * x - W;
    const int y0 = ty * 32 + (threadIdx.x >> 5);
    long long sx = cosq * X2 - sinq * (2LL * y0 - H) + ((long long)W << (MP_FIX_FRAC - 1));
    long long sy = sinq * X2 + cosq * (2LL * y0 - H) + ((long long)H << (MP_FIX_FRAC - 1));
    const long long stx = -16LL * sinq, sty = 16LL * cosq;   // y += 8
    const bool has_pro = J.pro.n > 0;
    const PwFast epi = mp_pw_fast(J.epi);
    const int xo = J.flip ? (J.wo - 1 - x) : x;
    float *dstb = J.dst;
    const int dp = J.dst_pitch;
#pragma unroll 1
    for (int i = 0; i < 4; ++i) {
        const int y = y0 + 8 * i;
        if (y < ho) {
            const int ix = (int)(sx >> MP_FIX_FRAC);
            const int iy = (int)(sy >> MP_FIX_FRAC);
            const float fx = (float)((int)(sx >> (MP_FIX_FRAC - 24)) & 0xFFFFFF) * 5.9604644775390625e-8f;
            const float fy = (float)((int)(sy >> (MP_FIX_FRAC - 24)) & 0xFFFFFF) * 5.9604644775390625e-8f;
            float a[4], b[4], c[4], d[4];
            if (!has_pro && (unsigned)ix < (unsigned)(W - 1) && (unsigned)iy < (unsigned)(H - 1)) {
                const float *p0 = src + (iy * sp + ix * CIN);
                const float *p1 = p0 + sp;
#pragma unroll
                for (int k = 0; k < CMID; ++k) {
                    a[k] = __ldg(p0 + k);
                    b[k] = __ldg(p0 + CIN + k);
                    c[k] = __ldg(p1 + k);
                    d[k] = __ldg(p1 + CIN + k);
                }
            } else {
                mp_load_px<CIN>(J, ix, iy, a);
                mp_load_px<CIN>(J, ix + 1, iy, b);
                mp_load_px<CIN>(J, ix, iy + 1, c);
                mp_load_px<CIN>(J, ix + 1, iy + 1, d);
            }
            float v[4] = {0.f, 0.f, 0.f, 0.f};
            const float gx = 1.0f - fx, gy = 1.0f - fy;
#pragma unroll
            for (int k = 0; k < CMID; ++k)
                v[k] = gy * (gx * a[k] + fx * b[k]) + fy * (gx * c[k] + fx * d[k]);
            float *drow = dstb + (size_t)y * dp;
            if (epi.n == 0) {
                float *o = drow + xo * CMID;
#pragma unroll
                for (int k = 0; k < CMID; ++k) o[k] = v[k];
            } else {
                const int co = mp_pw_apply_f(epi, J.epi, v, CMID);
                float *o = drow + xo * co;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (k < co) o[k] = v[k];
            }
        }
        sx += stx;
        sy += sty;
    }
}

// ---------------------------------------------------------------------------
// TRANSPOSE: 32x32 source tile through shared memory (+1 float row padding).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mp_transpose_tile(const MPJob &J, int t, float *tile)
{
    const int ty = t / J.tiles_x, tx = t - ty * J.tiles_x;
    const int x0 = tx * 32, y0 = ty * 32;           // source tile origin
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    const int cmid = J.cmid;
    const int ld = 32 * 4 + 1;
    for (int i = 0; i < 4; ++i) {
        const int y = y0 + ly + 8 * i, x = x0 + lx;
        float v[4] = {0.f, 0.f, 0.f, 0.f};
        if (x < J.w && y < J.h) {
            const float *p = J.src + (size_t)y * J.src_pitch + (size_t)x * J.cin;
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (c < J.cin) v[c] = __ldg(p + c);
            if (J.pro.n) mp_pw_apply(J.pro, v, J.cin);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
            if (c < cmid) tile[(ly + 8 * i) * ld + lx * cmid + c] = v[c];
    }
    __syncthreads();
    for (int i = 0; i < 4; ++i) {
        // output pixel (xo, yo) = source (yo, xo): output row = source column
        const int yo = x0 + ly + 8 * i, xo = y0 + lx;
        if (yo >= J.ho || xo >= J.wo) continue;
        float v[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) v[c] = (c < cmid) ? tile[lx * ld + (ly + 8 * i) * cmid + c] : 0.f;
        const int co = mp_pw_apply(J.epi, v, cmid);
        const int xf = J.flip ? (J.wo - 1 - xo) : xo;
        float *dst = J.dst + (size_t)yo * J.dst_pitch + (size_t)xf * co;
#pragma unroll
        for (int c = 0; c < 4; ++c)
            if (c < co) dst[c] = v[c];
    }
}

// ---------------------------------------------------------------------------
// POINT: 256 pixels x 4 rows per tile; prologue then epilogue, fliplr map.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mp_point_tile(const MPJob &J, int t)
{
    const int ty = t / J.tiles_x, tx = t - ty * J.tiles_x;
    const int x = tx * 256 + threadIdx.x;
    if (x >= J.w) return;
    for (int i = 0; i < 4; ++i) {
        const int y = ty * 4 + i;
        if (y >= J.h) break;
        const float *p = J.src + (size_t)y * J.src_pitch + (size_t)x * J.cin;
        float v[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int c = 0; c < 4; ++c)
            if (c < J.cin) v[c] = __ldg(p + c);
        int cc = mp_pw_apply(J.pro, v, J.cin);
        cc = mp_pw_apply(J.epi, v, cc);
        const int xo = J.flip ? (J.wo - 1 - x) : x;
        float *dst = J.dst + (size_t)y * J.dst_pitch + (size_t)xo * cc;
#pragma unroll
        for (int c = 0; c < 4; ++c)
            if (c < cc) dst[c] = v[c];
    }
}

// ---------------------------------------------------------------------------
// Kernel entry points.  Batch kernels read their image's job through a
// per-tile job index (one int load), single kernels take the job by value.
// ---------------------------------------------------------------------------
template <int KIND, int V>
__device__ __forceinline__ void mp_run_tile(const MPJob &J, int lt, bool map_in_global, int *err)
{
    extern __shared__ unsigned char mp_dyn_smem[];
    if (KIND == MPK_GAUSS) {
        mp_gauss_tile<MPChan<V>::CIN, MPChan<V>::CMID>(J, lt, mp_dyn_smem, map_in_global, err);
    } else if (KIND == MPK_ROTATE) {
        mp_rotate_tile<MPChan<V>::CIN, MPChan<V>::CMID>(J, lt);
    } else if (KIND == MPK_TRANSPOSE) {
        __shared__ float tile[32 * (32 * 4 + 1)];
        mp_transpose_tile(J, lt, tile);
    } else {
        mp_point_tile(J, lt);
    }
}

// Named wrappers, so profiles say which kernel ran.
#define MP_NAMED(NAME, KIND, V)                                                                    \
    __global__ void __launch_bounds__(MP_THREADS)                                                  \
        NAME##_batch(const MPJob *__restrict__ jobs, const int *__restrict__ tile_job, int *err)   \
    {                                                                                              \
        const int t = blockIdx.x;                                                                  \
        const MPJob &J = jobs[__ldg(tile_job + t)];                                                \
        mp_run_tile<KIND, V>(J, t - J.tile0, true, err);                                           \
    }                                                                                              \
    __global__ void __launch_bounds__(MP_THREADS)                                                  \
        NAME##_single(const __grid_constant__ MPJob job, int *err)                                 \
    {                                                                                              \
        mp_run_tile<KIND, V>(job, blockIdx.x, false, err);                                         \
    }
MP_NAMED(mp_rotate_c1, MPK_ROTATE, 0)
MP_NAMED(mp_rotate_c3, MPK_ROTATE, 1)
MP_NAMED(mp_rotate_c4, MPK_ROTATE, 2)
MP_NAMED(mp_rotate_grey3, MPK_ROTATE, 3)
MP_NAMED(mp_rotate_grey4, MPK_ROTATE, 4)
MP_NAMED(mp_transpose, MPK_TRANSPOSE, 0)
MP_NAMED(mp_point, MPK_POINT, 0)

// Gaussian kernels: one tile per CTA, 3 CTAs of 256 threads per SM fit in
// registers (80 per thread).
#define MP_GAUSS_NAMED(NAME, V)                                                                    \
    __global__ void __launch_bounds__(MP_THREADS, 3)                                               \
        NAME##_batch(const MPJob *__restrict__ jobs, const int *__restrict__ tile_job, int *err)   \
    {                                                                                              \
        const int t = blockIdx.x;                                                                  \
        const MPJob &J = jobs[__ldg(tile_job + t)];                                                \
        mp_run_tile<MPK_GAUSS, V>(J, t - J.tile0, true, err);                                      \
    }                                                                                              \
    __global__ void __launch_bounds__(MP_THREADS, 3)                                               \
        NAME##_single(const __grid_constant__ MPJob job, int *err)                                 \
    {                                                                                              \
        mp_run_tile<MPK_GAUSS, V>(job, blockIdx.x, false, err);                                    \
    }
MP_GAUSS_NAMED(mp_gauss_c1, 0)
MP_GAUSS_NAMED(mp_gauss_c3, 1)
MP_GAUSS_NAMED(mp_gauss_c4, 2)
MP_GAUSS_NAMED(mp_gauss_grey3, 3)
MP_GAUSS_NAMED(mp_gauss_grey4, 4)

// In-place channel-agnostic pointwise list (brightness, gamma) over a flat
// float buffer: float4 body plus scalar tail.
__global__ void __launch_bounds__(MP_THREADS) mp_k_flat(float *__restrict__ data, size_t n,
                                                        const __grid_constant__ PwList L)
{
    const size_t n4 = n / 4;
    float4 *d4 = reinterpret_cast<float4 *>(data);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4;
         i += (size_t)gridDim.x * blockDim.x) {
        float4 q = d4[i];
        float v0[4] = {q.x, 0.f, 0.f, 0.f}, v1[4] = {q.y, 0.f, 0.f, 0.f};
        float v2[4] = {q.z, 0.f, 0.f, 0.f}, v3[4] = {q.w, 0.f, 0.f, 0.f};
        mp_pw_apply(L, v0, 1);
        mp_pw_apply(L, v1, 1);
        mp_pw_apply(L, v2, 1);
        mp_pw_apply(L, v3, 1);
        d4[i] = make_float4(v0[0], v1[0], v2[0], v3[0]);
    }
    const size_t tail = n4 * 4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (tail < n) {
        float v[4] = {data[tail], 0.f, 0.f, 0.f};
        mp_pw_apply(L, v, 1);
        data[tail] = v[0];
    }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
// Raises a kernel's dynamic shared-memory limit to the device's opt-in
// maximum the first time a launch needs more than the 48 KB default.  The
// limit only ever grows, so launches prepared earlier stay valid.
static MPStatus mp_prepare_smem(const void *fn, size_t smem)
{
    if (smem <= 48 * 1024) return MILLIPYDE_SUCCESS;
    static std::mutex mtx;
    static std::vector<std::pair<const void *, int>> done;   // (kernel, device)
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mtx);
    for (auto &d : done)
        if (d.first == fn && d.second == dev) return MILLIPYDE_SUCCESS;
    int optin = 0;
    cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return mp_cuda_status(e);
    if ((size_t)optin < smem) return MP_ERROR_TOO_LARGE;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e != cudaSuccess) return mp_cuda_status(e);
    done.push_back({fn, dev});
    return MILLIPYDE_SUCCESS;
}

static int mp_current_device()
{
    int d = 0;
    cudaGetDevice(&d);
    return d;
}

int mp_variant(int cin, int cmid)
{
    if (cin == 1 && cmid == 1) return 0;
    if (cin == 3 && cmid == 3) return 1;
    if (cin == 4 && cmid == 4) return 2;
    if (cin == 3 && cmid == 1) return 3;
    if (cin == 4 && cmid == 1) return 4;
    return -1;
}

static const void *mp_batch_fn(int kind, int v)
{
    static const void *gauss[5] = {(const void *)mp_gauss_c1_batch, (const void *)mp_gauss_c3_batch,
                                   (const void *)mp_gauss_c4_batch, (const void *)mp_gauss_grey3_batch,
                                   (const void *)mp_gauss_grey4_batch};
    static const void *rot[5] = {(const void *)mp_rotate_c1_batch, (const void *)mp_rotate_c3_batch,
                                 (const void *)mp_rotate_c4_batch, (const void *)mp_rotate_grey3_batch,
                                 (const void *)mp_rotate_grey4_batch};
    switch (kind) {
    case MPK_GAUSS: return (v >= 0 && v < 5) ? gauss[v] : nullptr;
    case MPK_ROTATE: return (v >= 0 && v < 5) ? rot[v] : nullptr;
    case MPK_TRANSPOSE: return (const void *)mp_transpose_batch;
    default: return (const void *)mp_point_batch;
    }
}

static const void *mp_single_fn(int kind, int v)
{
    static const void *gauss[5] = {(const void *)mp_gauss_c1_single, (const void *)mp_gauss_c3_single,
                                   (const void *)mp_gauss_c4_single, (const void *)mp_gauss_grey3_single,
                                   (const void *)mp_gauss_grey4_single};
    static const void *rot[5] = {(const void *)mp_rotate_c1_single, (const void *)mp_rotate_c3_single,
                                 (const void *)mp_rotate_c4_single, (const void *)mp_rotate_grey3_single,
                                 (const void *)mp_rotate_grey4_single};
    switch (kind) {
    case MPK_GAUSS: return (v >= 0 && v < 5) ? gauss[v] : nullptr;
    case MPK_ROTATE: return (v >= 0 && v < 5) ? rot[v] : nullptr;
    case MPK_TRANSPOSE: return (const void *)mp_transpose_single;
    default: return (const void *)mp_point_single;
    }
}

MPStatus mp_prepare_kind(int kind, int variant, size_t smem)
{
    const void *fn = mp_batch_fn(kind, variant);
    if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
    MPStatus st = mp_prepare_smem(fn, smem);
    if (st != MILLIPYDE_SUCCESS) return st;
    return MILLIPYDE_SUCCESS;
}

// Kernel launch only (no allocation, no attribute change), so it may be
// captured into a CUDA graph; mp_prepare_kind must have run for the launch.
// `gauss` carries the tile geometry of GAUSS launches.
MPStatus mp_launch_kind(int kind, int variant, const MPJob *jobs_dev, const int *tile_job,
                        int total_tiles, size_t smem, int *err, cudaStream_t s, const int *gauss)
{
    if (total_tiles <= 0) return MILLIPYDE_SUCCESS;
    const void *fn = mp_batch_fn(kind, variant);
    if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
    (void)gauss;
    void *args[] = {(void *)&jobs_dev, (void *)&tile_job, (void *)&err};
    return mp_cuda_status(
        cudaLaunchKernel(fn, dim3(total_tiles), dim3(MP_THREADS), args, smem, s));
}

static MPStatus mp_launch_single_impl(int kind, const MPJob &job, size_t smem, int *err, cudaStream_t s)
{
    if (job.ntiles <= 0) return MILLIPYDE_SUCCESS;
    const void *fn = mp_single_fn(kind, mp_variant(job.cin, job.cmid));
    if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
    MPStatus st = mp_prepare_smem(fn, smem);
    if (st != MILLIPYDE_SUCCESS) return st;
    void *args[] = {(void *)&job, (void *)&err};
    return mp_cuda_status(cudaLaunchKernel(fn, dim3(job.ntiles), dim3(MP_THREADS), args, smem, s));
}

MPStatus mp_launch_single(int kind, const MPJob &job, size_t smem, cudaStream_t s)
{
    int *err = mp_device_error_word(mp_current_device());
    if (!err) return MP_ERROR_NO_DEVICE;
    return mp_launch_single_impl(kind, job, smem, err, s);
}

// Single-job launch reporting into a caller-supplied device error word
// (allocation-free path: nothing here allocates device memory).
MPStatus mp_launch_single_err(int kind, const MPJob &job, size_t smem, int *err, cudaStream_t s)
{
    return mp_launch_single_impl(kind, job, smem, err, s);
}

MPStatus mp_launch_flat(float *data, size_t n, const PwList &L, cudaStream_t s)
{
    if (n == 0) return MILLIPYDE_SUCCESS;
    size_t blocks = (n / 4 + MP_THREADS - 1) / MP_THREADS;
    if (blocks < 1) blocks = 1;
    if (blocks > 152 * 16) blocks = 152 * 16;
    mp_k_flat<<<(unsigned)blocks, MP_THREADS, 0, s>>>(data, n, L);
    return mp_cuda_status(cudaGetLastError());
}
