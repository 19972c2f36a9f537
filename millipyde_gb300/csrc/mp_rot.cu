// mp_rot.cu -- the footprint-staged bilinear rotate (sm_103a).
//
// Same operator and the same arithmetic as the ROTATE tile kernel: output
// pixel p samples the source at s = R(theta) (p - c) + c, c = (W/2, H/2)
// (the reference's geometry, src/millipyde_image.cpp:114-139), with s in
// 64-bit fixed point (MP_FIX_FRAC fractional bits) and the bilinear
// fractions taken from its top 23 fractional bits (the tile kernel and the
// rotate adjoint use 24; the difference, below 1.2e-7 of a pixel, is far
// inside the float32 tolerance); neighbours outside the source contribute 0.
// Each thread's first sample position is computed exactly as the tile
// kernel does; the following ones are stepped in 32-bit fixed point.
//
// What changes is where the neighbours come from.  For each TW x TH output
// tile the kernel works out the source footprint (the bounding box of the
// rotated tile plus the bilinear neighbour) and TMA copies that box into
// shared memory; boxes that leave the source arrive as zeros, which is the
// zero fill, so the gather has no bounds checks at all.  CTAs are
// persistent and double-buffered: the footprint of a CTA's next tile is in
// flight while the current one is sampled.
#include <mutex>
#include <utility>
#include <vector>

#include "mp_internal.cuh"

namespace {

// Footprint box origin (pixels) of output tile lt of job J.
__device__ __forceinline__ void ro_origin(const MPJob &J, int lt, int TW, int TH, int *bx, int *by, int *x0,
                                          int *y0)
{
    const int ty = lt / J.tiles_x, tx = lt - ty * J.tiles_x;
    *x0 = tx * TW;
    *y0 = ty * TH;
    const long long W = J.w, H = J.h;
    const long long xa = 2LL * *x0 - W, xb = 2LL * (*x0 + TW - 1) - W;
    const long long ya = 2LL * *y0 - H, yb = 2LL * (*y0 + TH - 1) - H;
    const long long cq = J.cosq, sq = J.sinq;
    // min over the four corners of sx = cq*X2 - sq*Y2 and sy = sq*X2 + cq*Y2
    const long long sx_min = min(cq * xa, cq * xb) + min(-sq * ya, -sq * yb) + (W << (MP_FIX_FRAC - 1));
    const long long sy_min = min(sq * xa, sq * xb) + min(cq * ya, cq * yb) + (H << (MP_FIX_FRAC - 1));
    // one pixel of margin before the footprint: the stepped positions may
    // drift below the exact ones by a few 2^-24 pixel
    *bx = (int)(sx_min >> MP_FIX_FRAC) - 1;
    *by = (int)(sy_min >> MP_FIX_FRAC) - 1;
}

// Kernel modes: the forward rotate; the adjoint's dx = R^T g (tiles of the
// source image, boxes of g); the adjoint's d theta (output tiles, boxes of
// the source, as the forward).
enum { RO_FWD = 0, RO_ADJ = 1, RO_DTH = 2 };

// Box origin (pixels) of source tile lt in the adjoint: the output pixels
// whose samples can use the tile's pixels lie around R(-theta)(q - c) + c;
// two pixels of margin before the exact minimum (the candidate window starts
// one pixel before the float position, which may round below the exact one).
__device__ __forceinline__ void ro_origin_adj(const MPJob &J, int lt, int TW, int TH, int *bx, int *by, int *x0,
                                              int *y0)
{
    const int ty = lt / J.tiles_x, tx = lt - ty * J.tiles_x;
    *x0 = tx * TW;
    *y0 = ty * TH;
    const long long W = J.w, H = J.h;
    const long long xa = 2LL * *x0 - W, xb = 2LL * (*x0 + TW - 1) - W;
    const long long ya = 2LL * *y0 - H, yb = 2LL * (*y0 + TH - 1) - H;
    const long long cq = J.cosq, sq = J.sinq;
    // min over the four corners of px = cq*X2 + sq*Y2 and py = -sq*X2 + cq*Y2
    const long long px_min = min(cq * xa, cq * xb) + min(sq * ya, sq * yb) + (W << (MP_FIX_FRAC - 1));
    const long long py_min = min(-sq * xa, -sq * xb) + min(cq * ya, cq * yb) + (H << (MP_FIX_FRAC - 1));
    *bx = (int)(px_min >> MP_FIX_FRAC) - 2;
    *by = (int)(py_min >> MP_FIX_FRAC) - 2;
}

// Per-buffer tile record written by the issuing thread: footprint origin
// (pixels), output tile origin, and the job fields the tile's threads use.
// The job table lives in global memory and the footprint buffers leave
// little L1 beside them, so reading the fields there cost each tile an L2
// round trip; the issuing thread copies them here one tile ahead.
struct RoTile {
    int bx, by, x0, y0;
    int jidx;                  // job of the tile (batch launches)
    int w, h, wo, ho, bxw, dp, flip;
    int en, eop;               // epilogue length and first op
    float e0, e1, e2;          // first op's parameters
    long long cq, sq;
    float *dst;
};
static_assert(sizeof(RoTile) <= 112, "two tile records must fit below the footprint buffers");

template <int C, int MODE = RO_FWD>
__device__ __forceinline__ void ro_issue(const MPJob &J, int jidx, int lt, float *buf, uint64_t *bar, RoTile *rec)
{
    int bx, by, x0, y0;
    if (MODE == RO_ADJ) ro_origin_adj(J, lt, mp_ro_tw(C), mp_ro_th(C), &bx, &by, &x0, &y0);
    else ro_origin(J, lt, mp_ro_tw(C), mp_ro_th(C), &bx, &by, &x0, &y0);
    rec->bx = bx;
    rec->by = by;
    rec->x0 = x0;
    rec->y0 = y0;
    rec->jidx = jidx;
    rec->w = J.w;
    rec->h = J.h;
    rec->wo = J.wo;
    rec->ho = J.ho;
    rec->bxw = J.bxw;
    rec->dp = J.dst_pitch;
    rec->flip = J.flip;
    rec->en = J.epi.n;
    rec->eop = J.epi.n ? J.epi.op[0].op : 0;
    rec->e0 = J.epi.op[0].p0;
    rec->e1 = J.epi.op[0].p1;
    rec->e2 = J.epi.op[0].p2;
    rec->cq = J.cosq;
    rec->sq = J.sinq;
    rec->dst = J.dst;
    const int xf = bx * C;
    mp_mbar_arrive_expect_tx(bar, (uint32_t)(J.bxw * J.byh * 4));
    mp_tma_load_2d(buf, &J.tmap, bar, xf & ~3, by);
}

// Packed float pairs (one f32x2 instruction each).
__device__ __forceinline__ float2 ro_fma2(float2 a, float2 b, float2 c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;"
        : "=l"(d)
        : "l"(*reinterpret_cast<unsigned long long *>(&a)), "l"(*reinterpret_cast<unsigned long long *>(&b)),
          "l"(*reinterpret_cast<unsigned long long *>(&c)));
    return *reinterpret_cast<float2 *>(&d);
}

__device__ __forceinline__ float2 ro_sub2(float2 a, float2 b)
{
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;"
        : "=l"(d)
        : "l"(*reinterpret_cast<unsigned long long *>(&a)), "l"(*reinterpret_cast<unsigned long long *>(&b)));
    return *reinterpret_cast<float2 *>(&d);
}

// Bilinear fraction of an 8.24 fixed-point coordinate from its top 23
// fractional bits: 2^23 + f23 as a float bit pattern (exact), scaled on the
// FMA pipe.
__device__ __forceinline__ float ro_frac_bits(int l) { return __int_as_float(0x4B000000 | ((l >> 1) & 0x7FFFFF)); }

// Epilogue kinds a tile is compiled for: none, one channel-preserving op of
// a known kind, or a general list.
enum { RO_EPI_NONE = 0, RO_EPI_GAMMA = 1, RO_EPI_BRIGHT = 2, RO_EPI_ONE = 3, RO_EPI_LIST = 4 };

// One output tile: every thread samples TW*TH/NT pixels, one column, rows
// NT/TW apart; the epilogue kind EK is decided once per tile.
template <int C, int EK>
__device__ __forceinline__ void ro_tile_k(const MPJob &J, const RoTile &T, const float *buf)
{
    constexpr int TW = mp_ro_tw(C), TH = mp_ro_th(C), NT = MP_RO_NT;
    constexpr int RSTEP = NT / TW, NPX = TW * TH / NT;
    const int bx = T.bx, by = T.by, x0 = T.x0, y0 = T.y0;
    const int delta = bx * C - ((bx * C) & ~3);
    const int bxw = T.bxw;
    const int x = x0 + (threadIdx.x & (TW - 1));
    const int yf = y0 + threadIdx.x / TW;
    const int wo = T.wo, ho = T.ho;
    if (x >= wo) return;
    const long long W = T.w, H = T.h, cq = T.cq, sq = T.sq;
    const long long X2 = 2LL * x - W, Y2 = 2LL * yf - H;
    // sample position relative to the box origin: exact in MP_FIX_FRAC fixed
    // point for the thread's first pixel, then stepped in 8.24 fixed point
    // (the step rounded down; the drift over NPX steps stays below
    // NPX * 2^-24 pixel)
    const long long rx0 = cq * X2 - sq * Y2 + (W << (MP_FIX_FRAC - 1)) - ((long long)bx << MP_FIX_FRAC);
    const long long ry0 = sq * X2 + cq * Y2 + (H << (MP_FIX_FRAC - 1)) - ((long long)by << MP_FIX_FRAC);
    int lx = (int)(rx0 >> (MP_FIX_FRAC - 24)), ly = (int)(ry0 >> (MP_FIX_FRAC - 24));
    const int stx = (int)((-2LL * RSTEP * sq) >> (MP_FIX_FRAC - 24));
    const int sty = (int)((2LL * RSTEP * cq) >> (MP_FIX_FRAC - 24));
    const float e0 = T.e0, e1 = T.e1, e2 = T.e2;
    const int dp = T.dp;
    const int xo = T.flip ? (wo - 1 - x) : x;
    float *drow = T.dst + (size_t)yf * dp + (size_t)xo * C;
    const size_t rstride = (size_t)RSTEP * dp;
    const bool full = y0 + TH <= ho;
    if constexpr (C == 1 && (EK == RO_EPI_NONE || EK == RO_EPI_GAMMA || EK == RO_EPI_BRIGHT)) {
        // one channel: two pixels (rows RSTEP apart) per step in packed
        // pairs; lerp as a + f (b - a)
        const float2 sc = make_float2(1.1920928955078125e-7f, 1.1920928955078125e-7f);
        const float2 m1 = make_float2(-1.0f, -1.0f);
#pragma unroll
        for (int i = 0; i < NPX; i += 2) {
            const int lxb = lx + stx, lyb = ly + sty;
            const float2 fx = ro_fma2(make_float2(ro_frac_bits(lx), ro_frac_bits(lxb)), sc, m1);
            const float2 fy = ro_fma2(make_float2(ro_frac_bits(ly), ro_frac_bits(lyb)), sc, m1);
            const float *pa = buf + (ly >> 24) * bxw + (lx >> 24) + delta;
            const float *pb = buf + (lyb >> 24) * bxw + (lxb >> 24) + delta;
            const float2 a = make_float2(pa[0], pb[0]), b = make_float2(pa[1], pb[1]);
            const float2 c = make_float2(pa[bxw], pb[bxw]), d = make_float2(pa[bxw + 1], pb[bxw + 1]);
            const float2 v0 = ro_fma2(fx, ro_sub2(b, a), a);
            const float2 v1 = ro_fma2(fx, ro_sub2(d, c), c);
            const float2 v = ro_fma2(fy, ro_sub2(v1, v0), v0);
            float o0 = v.x, o1 = v.y;
            if (EK == RO_EPI_GAMMA) {
                o0 = mp_clamp01(e1 * __powf(o0, e0));
                o1 = mp_clamp01(e1 * __powf(o1, e0));
            } else if (EK == RO_EPI_BRIGHT) {
                o0 = mp_clamp01(o0 + e0);
                o1 = mp_clamp01(o1 + e0);
            }
            if (full || yf + RSTEP * i < ho) drow[0] = o0;
            if (full || yf + RSTEP * (i + 1) < ho) drow[rstride] = o1;
            lx = lxb + stx;
            ly = lyb + sty;
            drow += 2 * rstride;
        }
        return;
    }
#pragma unroll
    for (int i = 0; i < NPX; ++i) {
        if (full || yf + RSTEP * i < ho) {
            // bilinear fractions from the top 23 fractional bits, converted on
            // the FMA pipe: 2^23 + f23 as a float bit pattern, then scaled
            const float fx = fmaf(__int_as_float(0x4B000000 | ((lx >> 1) & 0x7FFFFF)), 1.1920928955078125e-7f, -1.0f);
            const float fy = fmaf(__int_as_float(0x4B000000 | ((ly >> 1) & 0x7FFFFF)), 1.1920928955078125e-7f, -1.0f);
            const float *p0 = buf + (ly >> 24) * bxw + (lx >> 24) * C + delta;
            const float *p1 = p0 + bxw;
            const float gx = 1.0f - fx, gy = 1.0f - fy;
            float v[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int k = 0; k < C; ++k)
                v[k] = gy * (gx * p0[k] + fx * p0[C + k]) + fy * (gx * p1[k] + fx * p1[C + k]);
            if (EK == RO_EPI_LIST) {
                // general list: the output may have fewer channels
                const int c2 = mp_pw_apply(J.epi, v, C);
                float *d = T.dst + (size_t)(yf + RSTEP * i) * dp + (size_t)xo * c2;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (k < c2) d[k] = v[k];
            } else {
#pragma unroll
                for (int k = 0; k < C; ++k) {
                    const bool colour = !(C == 4 && k == 3);   // alpha passes untouched
                    float o = v[k];
                    if (EK == RO_EPI_GAMMA && colour) o = mp_clamp01(e1 * __powf(o, e0));
                    else if (EK == RO_EPI_BRIGHT && colour) o = mp_clamp01(o + e0);
                    else if (EK == RO_EPI_ONE) o = mp_pw_chan(T.eop, e0, e1, e2, o, k, C);
                    drow[k] = o;
                }
            }
        }
        lx += stx;
        ly += sty;
        drow += rstride;
    }
}

template <int C>
__device__ __forceinline__ void ro_tile(const MPJob &J, const RoTile &T, const float *buf)
{
    const int n = T.en;
    const int op = T.eop;
    if (n == 0) ro_tile_k<C, RO_EPI_NONE>(J, T, buf);
    else if (n == 1 && op == MP_OP_ADJUST_GAMMA) ro_tile_k<C, RO_EPI_GAMMA>(J, T, buf);
    else if (n == 1 && op == MP_OP_BRIGHTNESS) ro_tile_k<C, RO_EPI_BRIGHT>(J, T, buf);
    else if (n == 1 && op != MP_OP_RGB2GREY) ro_tile_k<C, RO_EPI_ONE>(J, T, buf);
    else ro_tile_k<C, RO_EPI_LIST>(J, T, buf);
}

// Exact forward sample position of output pixel (x, y) in MP_FIX_FRAC
// fixed point (the tile kernel's and the adjoint's arithmetic).
__device__ __forceinline__ void ro_src_fixed(const MPJob &J, int x, int y, long long &sx, long long &sy)
{
    const long long W = J.w, H = J.h;
    const long long X2 = 2LL * x - W, Y2 = 2LL * y - H;
    sx = J.cosq * X2 - J.sinq * Y2 + (W << (MP_FIX_FRAC - 1));
    sy = J.sinq * X2 + J.cosq * Y2 + (H << (MP_FIX_FRAC - 1));
}

__device__ __forceinline__ float ro_frac24(long long s)
{
    return (float)((int)((s >> (MP_FIX_FRAC - 24)) & 0xFFFFFF)) * 5.9604644775390625e-8f;
}

// Adjoint dx(q) = sum over output pixels p of w(p, q) g(p) for the pixels q
// of one source tile: each q visits the 4 x 4 output pixels around
// R(-theta)(q - c) + c, keeps those whose forward sample used q and applies
// the forward's bilinear weight (positions exact in fixed point, stepped by
// 2 cos / 2 sin: the map is affine).  g comes from the staged box; a
// candidate outside it (not expected) is read from global memory.  The job's
// source is g, its destination dx.
template <int C>
__device__ __forceinline__ void ro_adj_tile(const MPJob &J, const RoTile &T, const float *buf)
{
    constexpr int TW = mp_ro_tw(C), TH = mp_ro_th(C), NT = MP_RO_NT;
    constexpr int RSTEP = NT / TW, NPX = TW * TH / NT;
    const int bx = T.bx, by = T.by;
    const int delta = bx * C - ((bx * C) & ~3);
    const int bxw = J.bxw, bpx = (bxw - delta) / C, bh = J.byh;
    const int qx = T.x0 + (threadIdx.x & (TW - 1));
    const int qy0 = T.y0 + threadIdx.x / TW;
    const int W = J.w, H = J.h;
    if (qx >= W) return;
    const float hw = 0.5f * (float)W, hh = 0.5f * (float)H;
    const float ct = J.cth, st = J.sth;
    const long long c2 = 2 * J.cosq, s2 = 2 * J.sinq;
    const float *g = J.src;
    const int gp = J.src_pitch, dp = J.dst_pitch;
#pragma unroll 1
    for (int i = 0; i < NPX; ++i) {
        const int qy = qy0 + RSTEP * i;
        if (qy >= H) break;
        const float dxq = (float)qx - hw, dyq = (float)qy - hh;
        const int px0 = (int)floorf(ct * dxq + st * dyq + hw) - 1;
        const int py0 = (int)floorf(-st * dxq + ct * dyq + hh) - 1;
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        long long sxr, syr;
        ro_src_fixed(J, px0, py0, sxr, syr);
        // candidates in 8.24 fixed point relative to q: each row starts from
        // its exact position, the 4 candidates of a row step by the rounded
        // 8.24 step (drift below 3 * 2^-24 pixel)
        const long long qxf = (long long)qx << MP_FIX_FRAC, qyf = (long long)qy << MP_FIX_FRAC;
        const int c2s = (int)(c2 >> (MP_FIX_FRAC - 24)), s2s = (int)(s2 >> (MP_FIX_FRAC - 24));
#pragma unroll
        for (int jy = 0; jy < 4; ++jy) {
            const int py = py0 + jy;
            const bool yok = py >= 0 && py < H;
            int lx = (int)((sxr - qxf) >> (MP_FIX_FRAC - 24)), ly = (int)((syr - qyf) >> (MP_FIX_FRAC - 24));
#pragma unroll
            for (int jx = 0; jx < 4; ++jx) {
                const int px = px0 + jx;
                // floor(s) - q is -1 or 0 when q is one of the sample's neighbours
                const int ex = -(lx >> 24), ey = -(ly >> 24);
                if (yok && px >= 0 && px < W && (unsigned)ex <= 1u && (unsigned)ey <= 1u) {
                    const float fx = (float)(lx & 0xFFFFFF) * 5.9604644775390625e-8f;
                    const float fy = (float)(ly & 0xFFFFFF) * 5.9604644775390625e-8f;
                    const float w = (ey ? fy : 1.0f - fy) * (ex ? fx : 1.0f - fx);
                    const int ox = px - bx, oy = py - by;
                    if ((unsigned)ox < (unsigned)bpx && (unsigned)oy < (unsigned)bh) {
                        const float *v = buf + oy * bxw + ox * C + delta;
#pragma unroll
                        for (int c = 0; c < C; ++c) acc[c] = fmaf(w, v[c], acc[c]);
                    } else {
                        const float *v = g + (size_t)py * gp + (size_t)px * C;
#pragma unroll
                        for (int c = 0; c < C; ++c) acc[c] = fmaf(w, __ldg(v + c), acc[c]);
                    }
                }
                lx += c2s;
                ly += s2s;
            }
            sxr -= s2;
            syr += c2;
        }
        float *d = J.dst + (size_t)qy * dp + (size_t)qx * C;
#pragma unroll
        for (int c = 0; c < C; ++c) d[c] = acc[c];
    }
}

// Adjoint d theta over one output tile: sum over its pixels p of
// g(p) . (d bilinear(x, s) / d s) . (d s / d theta), s = R(theta)(p - c) + c,
// with x's neighbours from the staged box exactly as the forward reads them
// and g (J.aux, output layout) from global memory.  Returns this thread's
// share.
template <int C>
__device__ __forceinline__ float ro_dth_tile(const MPJob &J, const RoTile &T, const float *buf)
{
    constexpr int TW = mp_ro_tw(C), TH = mp_ro_th(C), NT = MP_RO_NT;
    constexpr int RSTEP = NT / TW, NPX = TW * TH / NT;
    const int bx = T.bx, by = T.by, x0 = T.x0, y0 = T.y0;
    const int delta = bx * C - ((bx * C) & ~3);
    const int bxw = J.bxw;
    const int x = x0 + (threadIdx.x & (TW - 1));
    const int yf = y0 + threadIdx.x / TW;
    const int wo = J.wo, ho = J.ho;
    if (x >= wo) return 0.f;
    const long long W = J.w, H = J.h, cq = J.cosq, sq = J.sinq;
    const long long X2 = 2LL * x - W, Y2 = 2LL * yf - H;
    const long long rx0 = cq * X2 - sq * Y2 + (W << (MP_FIX_FRAC - 1)) - ((long long)bx << MP_FIX_FRAC);
    const long long ry0 = sq * X2 + cq * Y2 + (H << (MP_FIX_FRAC - 1)) - ((long long)by << MP_FIX_FRAC);
    int lx = (int)(rx0 >> (MP_FIX_FRAC - 24)), ly = (int)(ry0 >> (MP_FIX_FRAC - 24));
    const int stx = (int)((-2LL * RSTEP * sq) >> (MP_FIX_FRAC - 24));
    const int sty = (int)((2LL * RSTEP * cq) >> (MP_FIX_FRAC - 24));
    const float hw = 0.5f * (float)W, hh = 0.5f * (float)H;
    const float ct = J.cth, st = J.sth;
    const float dxq = (float)x - hw;
    const float *gcol = J.aux + (size_t)x * C;
    float dth = 0.f;
#pragma unroll 4
    for (int i = 0; i < NPX; ++i) {
        const int y = yf + RSTEP * i;
        if (y < ho) {
            const float fx = fmaf(__int_as_float(0x4B000000 | ((lx >> 1) & 0x7FFFFF)), 1.1920928955078125e-7f, -1.0f);
            const float fy = fmaf(__int_as_float(0x4B000000 | ((ly >> 1) & 0x7FFFFF)), 1.1920928955078125e-7f, -1.0f);
            const float *p0 = buf + (ly >> 24) * bxw + (lx >> 24) * C + delta;
            const float *p1 = p0 + bxw;
            const float gx = 1.0f - fx, gy = 1.0f - fy;
            const float dyq = (float)y - hh;
            const float dsx = (-st * dxq - ct * dyq) * 0.01745329252f;
            const float dsy = (ct * dxq - st * dyq) * 0.01745329252f;
            const float *gp = gcol + (size_t)y * J.aux_pitch;
#pragma unroll
            for (int k = 0; k < C; ++k) {
                const float a = p0[k], b = p0[C + k], c = p1[k], d = p1[C + k];
                const float dvx = gy * (b - a) + fy * (d - c);
                const float dvy = gx * (c - a) + fx * (d - b);
                dth = fmaf(__ldg(gp + k), dvx * dsx + dvy * dsy, dth);
            }
        }
        lx += stx;
        ly += sty;
    }
    return dth;
}

__device__ __forceinline__ unsigned char *ro_base(unsigned char *smem_raw)
{
    return smem_raw + ((128 - (int)(mp_smem_addr(smem_raw) & 127)) & 127);
}

// Persistent loop over tiles t = first, first + step, ... of a tile -> job
// map (or of one job when `jobs` is null), warp-specialised: MP_RO_NT
// sampling threads and one producer warp whose lane 0 copies each tile's
// job fields into its record and issues its footprint's TMA.  Buffer k & 1
// holds tile k; `full` says its copy landed, `empty` that every sampling
// thread is done with it (each arrives after its tile's stores, or in the
// d theta mode after its running sum, which consume every value it loaded).
// No block-wide barrier: sampling warps never wait for the issuing
// thread's job-table reads or for each other; the d theta mode reduces its
// sums per warp (one FP64 atomic per warp when the CTA moves to another
// image).  Every wait is bounded; after a timeout the producer lets its
// copies in flight land before it returns.
template <int C, int MODE = RO_FWD>
__device__ __forceinline__ void ro_run_ws(const MPJob *jobs, const int *tile_job, const MPJob *one, int total,
                                          int buf_floats, int *err)
{
    extern __shared__ unsigned char mp_ro_smem[];
    unsigned char *base = ro_base(mp_ro_smem);
    uint64_t *full = reinterpret_cast<uint64_t *>(base);          // [2]
    uint64_t *empty = full + 2;                                    // [2]
    RoTile *recs = reinterpret_cast<RoTile *>(base + 32);         // one record per buffer
    float *bufs = reinterpret_cast<float *>(base + 256);
    if (threadIdx.x == 0) {
        mp_mbar_init(full, 1);
        mp_mbar_init(full + 1, 1);
        mp_mbar_init(empty, MP_RO_NT);
        mp_mbar_init(empty + 1, MP_RO_NT);
        mp_fence_barrier_init();
    }
    __syncthreads();
    const int first = blockIdx.x, step = gridDim.x;
    if (threadIdx.x >= MP_RO_NT) {
        if (threadIdx.x != MP_RO_NT) return;
        int k = 0;
        bool ok = true;
        for (int t = first; t < total; t += step, ++k) {
            const int b = k & 1;
            if (k >= 2 && !mp_mbar_wait_bounded(empty + b, (uint32_t)((k >> 1) - 1) & 1u)) {
                ok = false;
                break;
            }
            const int ji = one ? 0 : __ldg(tile_job + t);
            const MPJob &J = one ? *one : jobs[ji];
            if (!one) mp_tensormap_acquire(&J.tmap);
            ro_issue<C, MODE>(J, ji, one ? t : t - J.tile0, bufs + b * buf_floats, full + b, recs + b);
        }
        if (!ok) {
            atomicExch(err, MP_KERR_TIMEOUT);
            // tiles k - 2 and k - 1 were issued last (one per buffer)
            for (int q = k - 2; q < k; ++q)
                if (q >= 0) mp_mbar_wait_bounded(full + (q & 1), (uint32_t)(q >> 1) & 1u);
        }
        return;
    }
    // RO_DTH: this thread's running d theta share for job `cur`
    const MPJob *cur = nullptr;
    float dth = 0.f;
    auto flush = [&]() {
        float v = dth;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(cur->acc, (double)v);
        dth = 0.f;
    };
    int k = 0;
    for (int t = first; t < total; t += step, ++k) {
        const int b = k & 1;
        // the warp leaves together (the d theta mode shuffles across it)
        if (!__all_sync(0xffffffffu, mp_mbar_wait_bounded(full + b, (uint32_t)(k >> 1) & 1u))) {
            atomicExch(err, MP_KERR_TIMEOUT);
            return;
        }
        const RoTile rec = recs[b];
        const MPJob &J = one ? *one : jobs[rec.jidx];
        if (MODE == RO_FWD) {
            ro_tile<C>(J, rec, bufs + b * buf_floats);
            mp_mbar_arrive(empty + b);
        } else if (MODE == RO_ADJ) {
            ro_adj_tile<C>(J, rec, bufs + b * buf_floats);
            mp_mbar_arrive(empty + b);
        } else {
            if (cur != &J) {
                if (cur) flush();
                cur = &J;
            }
            dth += ro_dth_tile<C>(J, rec, bufs + b * buf_floats);
            mp_mbar_arrive_after(empty + b, dth);
        }
    }
    if (MODE == RO_DTH && cur) flush();
}

}  // namespace

#define MP_RO_KERNELS(NAME, C)                                                                       \
    __global__ void __launch_bounds__(MP_RO_NT_WS) NAME##_batch(const MPJob *__restrict__ jobs,    \
                                                                 const int *__restrict__ tile_job,  \
                                                                 int total, int buf_floats, int *err) \
    {                                                                                               \
        ro_run_ws<C>(jobs, tile_job, nullptr, total, buf_floats, err);                              \
    }                                                                                               \
    __global__ void __launch_bounds__(MP_RO_NT_WS)                                                 \
        NAME##_single(const __grid_constant__ MPJob job, int buf_floats, int *err)                  \
    {                                                                                               \
        ro_run_ws<C>(nullptr, nullptr, &job, job.ntiles, buf_floats, err);                          \
    }

MP_RO_KERNELS(mp_ro_c1, 1)
MP_RO_KERNELS(mp_ro_c3, 3)
MP_RO_KERNELS(mp_ro_c4, 4)

// The adjoint's modes (batch launches only).
#define MP_RO_MODE_KERNEL(NAME, C, MODE)                                                             \
    __global__ void __launch_bounds__(MP_RO_NT_WS, 4) NAME(const MPJob *__restrict__ jobs,           \
                                                        const int *__restrict__ tile_job, int total, \
                                                        int buf_floats, int *err)                    \
    {                                                                                               \
        ro_run_ws<C, MODE>(jobs, tile_job, nullptr, total, buf_floats, err);                         \
    }

MP_RO_MODE_KERNEL(mp_ro_adj_c1, 1, RO_ADJ)
MP_RO_MODE_KERNEL(mp_ro_adj_c3, 3, RO_ADJ)
MP_RO_MODE_KERNEL(mp_ro_adj_c4, 4, RO_ADJ)
MP_RO_MODE_KERNEL(mp_ro_dth_c1, 1, RO_DTH)
MP_RO_MODE_KERNEL(mp_ro_dth_c3, 3, RO_DTH)
MP_RO_MODE_KERNEL(mp_ro_dth_c4, 4, RO_DTH)

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
// Kernel of (mode, channel count); the adjoint's modes have batch kernels
// only (c + 8 * mode selects them).
static const void *mp_ro_fn(int c, bool single)
{
    switch (c) {
    case 1: return single ? (const void *)mp_ro_c1_single : (const void *)mp_ro_c1_batch;
    case 3: return single ? (const void *)mp_ro_c3_single : (const void *)mp_ro_c3_batch;
    case 4: return single ? (const void *)mp_ro_c4_single : (const void *)mp_ro_c4_batch;
    case 8 * RO_ADJ + 1: return single ? nullptr : (const void *)mp_ro_adj_c1;
    case 8 * RO_ADJ + 3: return single ? nullptr : (const void *)mp_ro_adj_c3;
    case 8 * RO_ADJ + 4: return single ? nullptr : (const void *)mp_ro_adj_c4;
    case 8 * RO_DTH + 1: return single ? nullptr : (const void *)mp_ro_dth_c1;
    case 8 * RO_DTH + 3: return single ? nullptr : (const void *)mp_ro_dth_c3;
    case 8 * RO_DTH + 4: return single ? nullptr : (const void *)mp_ro_dth_c4;
    default: return nullptr;
    }
}

size_t mp_ro_smem(int buf_floats) { return 256 + 2 * (size_t)buf_floats * 4 + 128; }

// Threads of a launch: the sampling threads plus the producer warp.
static int mp_ro_block(int) { return MP_RO_NT_WS; }

MPStatus mp_ro_prepare(int c, size_t smem, int *ctas_per_sm)
{
    static std::mutex mtx;
    static std::vector<std::pair<const void *, int>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return mp_cuda_status(e);
    for (int single = 0; single < 2; ++single) {
        const void *fn = mp_ro_fn(c, single != 0);
        if (!fn && single && c >= 8) continue;   // adjoint modes: batch kernel only
        if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
        std::lock_guard<std::mutex> lk(mtx);
        bool have = false;
        for (auto &d : done)
            if (d.first == fn && d.second == dev) have = true;
        if (have) continue;
        int optin = 0;
        e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return mp_cuda_status(e);
        // the opt-in maximum covers static and dynamic shared memory together
        cudaFuncAttributes fa;   // (static shared memory of the kernel)
        e = cudaFuncGetAttributes(&fa, fn);
        if (e != cudaSuccess) return mp_cuda_status(e);
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
        if (e != cudaSuccess) return mp_cuda_status(e);
        done.push_back({fn, dev});
    }
    if (ctas_per_sm) {
        int n = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, mp_ro_fn(c, false), mp_ro_block(c), smem);
        if (e != cudaSuccess) return mp_cuda_status(e);
        if (n < 1) return MP_ERROR_TOO_LARGE;
        *ctas_per_sm = n;
    }
    return MILLIPYDE_SUCCESS;
}

MPStatus mp_ro_launch(int c, const MPJob *jobs_dev, const int *tile_job, int total, int buf_floats, int grid,
                      int *err, cudaStream_t s)
{
    if (total <= 0) return MILLIPYDE_SUCCESS;
    const void *fn = mp_ro_fn(c, false);
    if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
    if (grid > total) grid = total;
    if (grid < 1) grid = 1;
    void *args[] = {(void *)&jobs_dev, (void *)&tile_job, (void *)&total, (void *)&buf_floats, (void *)&err};
    return mp_cuda_status(cudaLaunchKernel(fn, dim3(grid), dim3(mp_ro_block(c)), args, mp_ro_smem(buf_floats), s));
}

MPStatus mp_ro_launch_single(int c, const MPJob &job, int buf_floats, int grid, int *err, cudaStream_t s)
{
    if (job.ntiles <= 0) return MILLIPYDE_SUCCESS;
    const void *fn = mp_ro_fn(c, true);
    if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
    if (grid > job.ntiles) grid = job.ntiles;
    if (grid < 1) grid = 1;
    void *args[] = {(void *)&job, (void *)&buf_floats, (void *)&err};
    return mp_cuda_status(cudaLaunchKernel(fn, dim3(grid), dim3(mp_ro_block(c)), args, mp_ro_smem(buf_floats), s));
}
