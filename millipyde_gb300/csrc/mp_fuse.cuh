// mp_fuse.cuh -- gaussian followed by rotate in one kernel (sm_103a), with
// the blurred image kept in shared memory.
//
// Same operators and arithmetic as the two kernels it replaces: the
// zero-padded separable gaussian with normalised taps, radius ceil(3 sigma)
// (the reference's weights and padding, src/millipyde_image.cpp:745-756,
// :170-172), then the bilinear rotate about (W/2, H/2) with zero fill
// (geometry of src/millipyde_image.cpp:114-139) in MP_FIX_FRAC fixed point
// as in mp_rot.cu.  The blur runs on one channel: a 1-channel source, or a
// 3- / 4-channel source whose prologue ends in rgb2grey.
//
// Per 64 x 64 output tile of the rotate:
//   footprint  the box of the blurred image the tile's bilinear samples read
//              (the rotated tile's bounding box plus the neighbour), bw x bh
//              pixels, and the source region that box needs for the blur:
//              (bw + 2R) x (bh + 2R);
//   stage      TMA copies of that region in chunks of 16 rows (boxes of 128
//              floats, double-buffered); boxes leaving the image arrive as
//              zeros;
//   prologue   each chunk row -> one value per pixel (rgb2grey / the
//              pointwise prologue) into the plane G; pixels outside the
//              image are 0 (the blur's zero padding);
//   vertical   G -> V: each thread owns two columns and slides a register
//              window of 8 + 2R rows down 24 output rows (packed f32x2
//              FMAs, symmetric taps), rows 2p and 2p + 1 interleaved in V;
//   horizontal V -> B: 8 outputs of two rows per work item, one f32x2 FMA
//              per tap for both rows; the gaussian's epilogue is applied and
//              pixels outside the image are set to 0 (the rotate's zero
//              fill);
//   gather     the rotate's bilinear samples from B, the rotate's epilogue
//              and the fliplr map, stored to global memory.
// V reuses the staging area and B the plane G.  The radius is a
// compile-time parameter (one instance per radius 1..12).
#pragma once
#include "mp_vh.cuh"

namespace mp_fz {

constexpr int NT = 256;    // threads per CTA
constexpr int TW = 64;     // output tile (one channel)
constexpr int TH = 64;
constexpr int CR = MP_FZ_CR; // source rows per staged chunk
constexpr int BXF = 128;   // floats per TMA box row
constexpr int VG = 24;     // vertical-pass output rows per thread group
constexpr int NVG = 4;     // thread groups: 4 x 24 rows >= the tallest footprint
constexpr int RSTEP = NT / TW, NPX = TW * TH / NT;

using mp_vh::add2;
using mp_vh::fma2;
using mp_vh::ld4;

__device__ __forceinline__ float2 ld2(const float *p) { return *reinterpret_cast<const float2 *>(p); }

// Footprint origin (pixels of the blurred image) of output tile lt: the
// minimum over the tile's corners of the exact sample position, one pixel
// of margin (the rotate kernel's rule, mp_rot.cu).
__device__ __forceinline__ void fz_origin(const MPJob &J, int lt, int *bx, int *by, int *x0, int *y0)
{
    const int ty = lt / J.tiles_x, tx = lt - ty * J.tiles_x;
    *x0 = tx * TW;
    *y0 = ty * TH;
    const long long W = J.w, H = J.h;
    const long long xa = 2LL * *x0 - W, xb = 2LL * (*x0 + TW - 1) - W;
    const long long ya = 2LL * *y0 - H, yb = 2LL * (*y0 + TH - 1) - H;
    const long long cq = J.cosq, sq = J.sinq;
    const long long sx_min = min(cq * xa, cq * xb) + min(-sq * ya, -sq * yb) + (W << (MP_FIX_FRAC - 1));
    const long long sy_min = min(sq * xa, sq * xb) + min(cq * ya, cq * yb) + (H << (MP_FIX_FRAC - 1));
    *bx = (int)(sx_min >> MP_FIX_FRAC) - 1;
    *by = (int)(sy_min >> MP_FIX_FRAC) - 1;
}

__device__ __forceinline__ float fz_frac(int l) { return __int_as_float(0x4B000000 | ((l >> 1) & 0x7FFFFF)); }

enum { FZ_EPI_NONE = 0, FZ_EPI_GAMMA = 1, FZ_EPI_BRIGHT = 2, FZ_EPI_LIST = 3 };

// The rotate's bilinear gather from B (origin bx, by; pitch bp) for this
// thread's column of the tile: two pixels (rows RSTEP apart) per step in
// packed pairs, lerp as a + f (b - a), epilogue kind EK.
template <int EK>
__device__ __forceinline__ void fz_gather(const MPJob &J, const float *B, int bp, int bx, int by, int x0, int y0)
{
    const int x = x0 + (threadIdx.x & (TW - 1));
    const int yf = y0 + threadIdx.x / TW;
    const int wo = J.wo, ho = J.ho;
    if (x >= wo) return;
    const long long W = J.w, H = J.h, cq = J.cosq, sq = J.sinq;
    const long long X2 = 2LL * x - W, Y2 = 2LL * yf - H;
    const long long rx0 = cq * X2 - sq * Y2 + (W << (MP_FIX_FRAC - 1)) - ((long long)bx << MP_FIX_FRAC);
    const long long ry0 = sq * X2 + cq * Y2 + (H << (MP_FIX_FRAC - 1)) - ((long long)by << MP_FIX_FRAC);
    int lx = (int)(rx0 >> (MP_FIX_FRAC - 24)), ly = (int)(ry0 >> (MP_FIX_FRAC - 24));
    const int stx = (int)((-2LL * RSTEP * sq) >> (MP_FIX_FRAC - 24));
    const int sty = (int)((2LL * RSTEP * cq) >> (MP_FIX_FRAC - 24));
    const PwFast epi = mp_pw_fast(J.epi);
    const float e0 = epi.p0, e1 = epi.p1;
    const int dp = J.dst_pitch;
    const int xo = J.flip ? (wo - 1 - x) : x;
    float *drow = J.dst + (size_t)yf * dp + xo;
    const size_t rstride = (size_t)RSTEP * dp;
    const bool full = y0 + TH <= ho;
    const float2 sc = make_float2(1.1920928955078125e-7f, 1.1920928955078125e-7f);
    const float2 m1 = make_float2(-1.0f, -1.0f);
#pragma unroll
    for (int i = 0; i < NPX; i += 2) {
        const int lxb = lx + stx, lyb = ly + sty;
        const float2 fx = fma2(make_float2(fz_frac(lx), fz_frac(lxb)), sc, m1);
        const float2 fy = fma2(make_float2(fz_frac(ly), fz_frac(lyb)), sc, m1);
        const float *pa = B + (ly >> 24) * bp + (lx >> 24);
        const float *pb = B + (lyb >> 24) * bp + (lxb >> 24);
        const float2 a = make_float2(pa[0], pb[0]), b = make_float2(pa[1], pb[1]);
        const float2 c = make_float2(pa[bp], pb[bp]), d = make_float2(pa[bp + 1], pb[bp + 1]);
        const float2 v0 = fma2(fx, make_float2(b.x - a.x, b.y - a.y), a);
        const float2 v1 = fma2(fx, make_float2(d.x - c.x, d.y - c.y), c);
        const float2 v = fma2(fy, make_float2(v1.x - v0.x, v1.y - v0.y), v0);
        float o0 = v.x, o1 = v.y;
        if (EK == FZ_EPI_GAMMA) {
            o0 = mp_clamp01(e1 * __powf(o0, e0));
            o1 = mp_clamp01(e1 * __powf(o1, e0));
        } else if (EK == FZ_EPI_BRIGHT) {
            o0 = mp_clamp01(o0 + e0);
            o1 = mp_clamp01(o1 + e0);
        } else if (EK == FZ_EPI_LIST) {
            o0 = mp_pw_chan_f(epi, J.epi, o0, 0, 1);
            o1 = mp_pw_chan_f(epi, J.epi, o1, 0, 1);
        }
        if (full || yf + RSTEP * i < ho) drow[0] = o0;
        if (full || yf + RSTEP * (i + 1) < ho) drow[rstride] = o1;
        lx = lxb + stx;
        ly = lyb + sty;
        drow += 2 * rstride;
    }
}

// One output tile of job J with compiled radius R.  `chunks` counts the
// CTA's staged chunks (barrier phases); false after a timed-out wait (the
// error word is set and the copies in flight have landed).
template <int CIN, int R>
__device__ __noinline__ bool fz_tile(const MPJob &J, int lt, float *base, const FzGeom &g, uint32_t &chunks,
                                     int *err)
{
    constexpr int NTAP = 2 * R + 1;
    constexpr int NWIN = 8 + 2 * R;
    constexpr int NLD2 = (8 + 2 * R + 1) / 2;   // float4 loads (two columns of a row pair) per H item
    const int tid = threadIdx.x;
    uint64_t *bars = reinterpret_cast<uint64_t *>(base);
    float *stg = base + 32;
    float *V = stg;
    float *G = base + g.offG;
    float *B = G;
    const int gp = g.gp;

    int bx, by, x0, y0;
    fz_origin(J, lt, &bx, &by, &x0, &y0);
    const int bw = J.bxw, bh = J.byh;           // footprint box (pixels)
    const int sw = bw + 2 * R, sh = bh + 2 * R;  // source region of the blur
    const int sx0 = bx - R, sy0 = by - R;
    const int xf = sx0 * CIN, xa = xf & ~3, delta = xf - xa;
    const int nb = (delta + sw * CIN + BXF - 1) / BXF;
    const int nch = (sh + CR - 1) / CR;
    const int W = J.w, H = J.h;

    auto issue = [&](int c) {
        const uint32_t q = chunks + (uint32_t)c;
        uint64_t *bar = bars + (q & 1u);
        float *dst = stg + (q & 1u) * g.stage;
        mp_mbar_arrive_expect_tx(bar, (uint32_t)(nb * BXF * CR * 4));
        for (int b = 0; b < nb; ++b) mp_tma_load_2d(dst + b * BXF * CR, &J.tmap, bar, xa + BXF * b, sy0 + CR * c);
    };
    if (tid == 0) {
        mp_tensormap_acquire(&J.tmap);
        issue(0);
        if (nch > 1) issue(1);
    }

    // ---- stage + prologue: source region -> G (one value per pixel)
    const PwFast pro = mp_pw_fast(J.pro);
    const bool grey_only = CIN >= 3 && J.pro.n == 1 && pro.op == MP_OP_RGB2GREY;
    for (int c = 0; c < nch; ++c) {
        const uint32_t q = chunks + (uint32_t)c;
        const bool ok = mp_mbar_wait_bounded(bars + (q & 1u), (q >> 1) & 1u);
        if (!__syncthreads_and(ok)) {
            if (tid == 0) atomicExch(err, MP_KERR_TIMEOUT);
            for (int k = c; k < nch && k < c + 2; ++k) {
                const uint32_t qk = chunks + (uint32_t)k;
                mp_mbar_wait_bounded(bars + (qk & 1u), (qk >> 1) & 1u);
            }
            return false;
        }
        const float *sb = stg + (q & 1u) * g.stage;
        const int col = tid & 127;
        const int sxp = sx0 + col;
        const bool colin = col < sw && sxp >= 0 && sxp < W;
#pragma unroll
        for (int pass = 0; pass < CR / 2; ++pass) {
            const int rr = 2 * pass + (tid >> 7);
            const int gr = CR * c + rr;
            if (col < sw && gr < sh) {
                float v[4] = {0.f, 0.f, 0.f, 0.f};
                const float *sp = sb + rr * BXF;
#pragma unroll
                for (int k = 0; k < CIN; ++k) {
                    const int f = delta + col * CIN + k;
                    v[k] = sp[(f >> 7) * (BXF * CR) + (f & 127)];
                }
                float val;
                if (grey_only) val = fminf(1.0f, 0.2125f * v[0] + 0.7154f * v[1] + 0.0721f * v[2]);
                else {
                    mp_pw_apply_f(pro, J.pro, v, CIN);
                    val = v[0];
                }
                const int syp = sy0 + gr;
                G[gr * gp + col] = (colin && syp >= 0 && syp < H) ? val : 0.f;
            }
        }
        __syncthreads();   // stage q & 1 read (values stored to G), G rows written
        if (tid == 0 && c + 2 < nch) issue(c + 2);
    }
    chunks += (uint32_t)nch;

    // symmetric taps w[m] = w[2R - m], m = 0..R, as packed pairs
    float2 w2[R + 1];
#pragma unroll
    for (int m = 0; m <= R; ++m) {
        const float t = J.wts[m];
        w2[m] = make_float2(t, t);
    }

    // ---- vertical pass: G -> V (rows 2i, 2i + 1 interleaved per column)
    {
        const int p = tid & 63, qg = tid >> 6;
        const int c0 = 2 * p, o0 = VG * qg;
        if (c0 < sw && o0 < bh) {
            float2 win[NWIN];
            const float *gc = G + o0 * gp + c0;
#pragma unroll
            for (int j = 0; j < 2 * R; ++j) win[j] = ld2(gc + j * gp);
            float *vb = V + (o0 >> 1) * (2 * gp) + 2 * c0;
#pragma unroll
            for (int st = 0; st < VG / 8; ++st) {
#pragma unroll
                for (int j = 0; j < 8; ++j) win[2 * R + j] = ld2(gc + (2 * R + 8 * st + j) * gp);
                float2 prev = make_float2(0.f, 0.f);
#pragma unroll
                for (int o = 0; o < 8; ++o) {
                    float2 a = fma2(w2[R], win[o + R], make_float2(0.f, 0.f));
#pragma unroll
                    for (int k = 0; k < R; ++k) a = fma2(w2[k], add2(win[o + k], win[o + 2 * R - k]), a);
                    if (o & 1)
                        *reinterpret_cast<float4 *>(vb + (4 * st + (o >> 1)) * (2 * gp)) =
                            make_float4(prev.x, a.x, prev.y, a.y);
                    else
                        prev = a;
                }
#pragma unroll
                for (int j = 0; j < 2 * R; ++j) win[j] = win[j + 8];
            }
        }
    }
    __syncthreads();

    // ---- horizontal pass: V -> B, the gaussian's epilogue, zero outside
    //      the image (item = 8 outputs of rows 2 rp and 2 rp + 1)
    {
        const int npr = (bh + 1) >> 1, ngx = (bw + 7) >> 3;
        const PwFast mid = mp_pw_fast(J.epi2);
        for (int i = tid; i < 48 * 16; i += NT) {
            const int gx = i / 48, rp = i - gx * 48;
            if (rp >= npr || gx >= ngx) continue;
            const float *vp = V + rp * (2 * gp) + 16 * gx;
            float2 o2[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) o2[k] = make_float2(0.f, 0.f);
#pragma unroll
            for (int q = 0; q < NLD2; ++q) {
                const float4 v = ld4(vp + 4 * q);
                const float2 pc[2] = {make_float2(v.x, v.y), make_float2(v.z, v.w)};
#pragma unroll
                for (int u = 0; u < 2; ++u) {
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const int m = 2 * q + u - k;
                        if (m >= 0 && m < NTAP) o2[k] = fma2(w2[m <= R ? m : 2 * R - m], pc[u], o2[k]);
                    }
                }
            }
            const int xb0 = bx + 8 * gx;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int y = 2 * rp + h;
                const bool rin = (unsigned)(by + y) < (unsigned)H;
                float o[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    float t = h ? o2[k].y : o2[k].x;
                    if (mid.n) t = mp_pw_chan_f(mid, J.epi2, t, 0, 1);
                    o[k] = (rin && (unsigned)(xb0 + k) < (unsigned)W) ? t : 0.f;
                }
                float *bp_ = B + y * gp + 8 * gx;
                *reinterpret_cast<float4 *>(bp_) = make_float4(o[0], o[1], o[2], o[3]);
                *reinterpret_cast<float4 *>(bp_ + 4) = make_float4(o[4], o[5], o[6], o[7]);
            }
        }
    }
    __syncthreads();

    // ---- gather: the rotate's samples from B, epilogue, fliplr, store
    {
        const int n = J.epi.n, op = J.epi.op[0].op;
        if (n == 0) fz_gather<FZ_EPI_NONE>(J, B, gp, bx, by, x0, y0);
        else if (n == 1 && op == MP_OP_ADJUST_GAMMA) fz_gather<FZ_EPI_GAMMA>(J, B, gp, bx, by, x0, y0);
        else if (n == 1 && op == MP_OP_BRIGHTNESS) fz_gather<FZ_EPI_BRIGHT>(J, B, gp, bx, by, x0, y0);
        else fz_gather<FZ_EPI_LIST>(J, B, gp, bx, by, x0, y0);
    }
    // V (generic stores) shares the staging area the next tile's copies
    // write through the async proxy; B is read before G is rewritten
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    return true;
}

template <int CIN>
__device__ __forceinline__ bool fz_dispatch(const MPJob &J, int lt, float *base, const FzGeom &g, uint32_t &chunks,
                                            int *err)
{
    switch (J.radius) {
#define MP_FZ_CASE(RR) \
    case RR: return fz_tile<CIN, RR>(J, lt, base, g, chunks, err);
        MP_FZ_CASE(1) MP_FZ_CASE(2) MP_FZ_CASE(3) MP_FZ_CASE(4) MP_FZ_CASE(5) MP_FZ_CASE(6)
        MP_FZ_CASE(7) MP_FZ_CASE(8) MP_FZ_CASE(9) MP_FZ_CASE(10) MP_FZ_CASE(11) MP_FZ_CASE(12)
#undef MP_FZ_CASE
    default: return true;   // the planner sends no other radius here
    }
}

__device__ __forceinline__ float *fz_base(float4 *raw)
{
    unsigned char *p = reinterpret_cast<unsigned char *>(raw);
    return reinterpret_cast<float *>(p + ((128 - (int)(mp_smem_addr(p) & 127)) & 127));
}

}  // namespace mp_fz

// Persistent kernel: CTA b takes tiles b, b + grid, ... of the tile -> job map.
#define MP_FZ_KERNEL(NAME, CIN)                                                                      \
    __global__ void __launch_bounds__(mp_fz::NT, 2) NAME(const MPJob *__restrict__ jobs,             \
                                                        const int *__restrict__ tile_job, int total, \
                                                        const FzGeom g, int *err)             \
    {                                                                                               \
        extern __shared__ float4 mp_fz_dsmem4[];                                                    \
        float *base = mp_fz::fz_base(mp_fz_dsmem4);                                                 \
        if (threadIdx.x == 0) {                                                                     \
            uint64_t *bars = reinterpret_cast<uint64_t *>(base);                                    \
            mp_mbar_init(bars, 1);                                                                  \
            mp_mbar_init(bars + 1, 1);                                                              \
            mp_fence_barrier_init();                                                                \
        }                                                                                           \
        __syncthreads();                                                                            \
        uint32_t chunks = 0;                                                                        \
        for (int t = blockIdx.x; t < total; t += gridDim.x) {                                       \
            const MPJob &J = jobs[__ldg(tile_job + t)];                                             \
            if (!mp_fz::fz_dispatch<CIN>(J, t - J.tile0, base, g, chunks, err)) return;             \
        }                                                                                           \
    }
