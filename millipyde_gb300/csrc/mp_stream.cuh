// mp_stream.cuh -- the strip-streaming separable gaussian (sm_103a).
//
// Same operator as the GAUSS tile kernel (zero-padded separable correlation
// with normalised exp(-k^2 / 2 sigma^2) taps, radius ceil(3 sigma); the
// reference's weights and padding are src/millipyde_image.cpp:745-756 and
// :170-172, :218-221), organised for HBM streaming instead of tiles.
//
// A work item is a STRIP: SW output columns by RS output rows of one image.
// A CTA walks its strip top to bottom in blocks of RB = MP_GS_RB rows:
//   TMA  the source rows of the next blocks (strip plus a halo of R4 = R
//        rounded up to 4 pixels on each side) stream into a ring of NS
//        shared-memory stages; boxes that leave the image arrive as zeros,
//        which is the zero padding.  One mbarrier per stage.
//   P    prologue + de-interleave: every staged pixel goes through the
//        pointwise prologue (zero outside the image) into channel planes
//        G[c][row][x], four pixels per thread.
//   H    horizontal pass: eight consecutive outputs per thread from a G row
//        into a ring H[c][row][x] holding the last (L + 1) * RB rows,
//        L = ceil(2R / RB).  Ring rows below 2R are also written after the
//        ring, so every vertical window is one contiguous run of rows.
//   V    vertical pass: 2 columns x 4 rows per thread over the H ring, the
//        pointwise epilogue and the fliplr output map applied on the way
//        out, stored straight to global memory.
// R is the radius rounded up to a compiled bucket (exact up to 12, then 16
// and 24, the taps zero padded): the H and V passes are then fully unrolled
// with the taps in registers.  Larger radii run the same passes as loops.
// Each source row is loaded, prologued and horizontally filtered once per
// strip (plus 2R halo rows at the top of a strip), and the vertical pass has
// no halo columns.  CTAs are persistent: CTA b takes items b, b + grid, ...
#pragma once
#include "mp_internal.cuh"

namespace mp_gs {

template <int CIN> struct GsIn;
template <> struct GsIn<1> { static constexpr int QPB = 16, LGQPB = 4; };   // 64-float boxes
template <> struct GsIn<3> { static constexpr int QPB = 4, LGQPB = 2; };    // 48-float boxes
template <> struct GsIn<4> { static constexpr int QPB = 4, LGQPB = 2; };    // 64-float boxes

constexpr int mp_lg2(int v) { return v <= 1 ? 0 : 1 + mp_lg2(v / 2); }

template <int CIN, int CMID> struct GsC {
    static constexpr int SW = mp_gs_sw(CMID), NT = mp_gs_nt(CMID), RB = mp_gs_rb(CMID), HW = SW + 4;
    static constexpr int LGSW = mp_lg2(SW), LGRB = mp_lg2(RB);
};

__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4(float *p, float a, float b, float c, float d)
{
    *reinterpret_cast<float4 *>(p) = make_float4(a, b, c, d);
}

// Taps 0..N-1 of a zero-padded tap array in smem, into registers.
template <int N>
__device__ __forceinline__ void load_taps(const float *w, float *t)
{
#pragma unroll
    for (int j = 0; j < (N + 3) / 4; ++j) {
        const float4 q = ld4(w + 4 * j);
        t[4 * j] = q.x;
        t[4 * j + 1] = q.y;
        t[4 * j + 2] = q.z;
        t[4 * j + 3] = q.w;
    }
}

// ---- compiled-radius passes -------------------------------------------------
// Horizontal: o[k] = sum_m t[m] * g[E + k + m], k < 8, m < 2R + 1, where
// g is 16-byte aligned and E = R4 - R.
template <int R>
__device__ __forceinline__ void h_item(const float *gp, const float *t, float o[8])
{
    constexpr int R4 = (R + 3) & ~3, E = R4 - R, NTAP = 2 * R + 1;
    constexpr int NLD = (E + 8 + 2 * R + 3) / 4;
    float x[4 * NLD];
#pragma unroll
    for (int j = 0; j < NLD; ++j) {
        const float4 q = ld4(gp + 4 * j);
        x[4 * j] = q.x;
        x[4 * j + 1] = q.y;
        x[4 * j + 2] = q.z;
        x[4 * j + 3] = q.w;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) o[k] = 0.f;
#pragma unroll
    for (int m = 0; m < NTAP; ++m)
#pragma unroll
        for (int k = 0; k < 8; ++k) o[k] = fmaf(t[m], x[E + k + m], o[k]);
}

// Vertical: acc[o][k] = sum_m t[m] * h[(o + m) * HW + k], o < 4, k < 2.
template <int R, int HW>
__device__ __forceinline__ void v_item(const float *hp, const float *t, float acc[4][2])
{
    constexpr int NTAP = 2 * R + 1, NROW = 4 + 2 * R;
#pragma unroll
    for (int o = 0; o < 4; ++o) acc[o][0] = acc[o][1] = 0.f;
#pragma unroll
    for (int j = 0; j < NROW; ++j) {
        const float2 y = *reinterpret_cast<const float2 *>(hp + j * HW);
#pragma unroll
        for (int o = 0; o < 4; ++o) {
            const int m = j - o;
            if (m >= 0 && m < NTAP) {
                acc[o][0] = fmaf(t[m], y.x, acc[o][0]);
                acc[o][1] = fmaf(t[m], y.y, acc[o][1]);
            }
        }
    }
}

// ---- loop passes (radius beyond the compiled buckets) -------------------------
// Horizontal with taps carrying E leading zeros (n4 a multiple of 4).
__device__ __forceinline__ void hfma4(float o[8], const float4 &P, const float4 &Q, const float4 &R,
                                      const float4 &w)
{
    const float x[12] = {P.x, P.y, P.z, P.w, Q.x, Q.y, Q.z, Q.w, R.x, R.y, R.z, R.w};
    const float ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
        for (int k = 0; k < 8; ++k) o[k] = fmaf(ww[s], x[k + s], o[k]);
}

__device__ __forceinline__ void h_loop(const float *gp, const float *w, int n4, float o[8])
{
#pragma unroll
    for (int k = 0; k < 8; ++k) o[k] = 0.f;
    float4 A = ld4(gp), B = ld4(gp + 4), C = ld4(gp + 8), D;
    float4 Wc = ld4(w), Wn;
    int m = 0;
#define MP_HSTEP(P, Q, Rr, N)                 \
    {                                         \
        N = ld4(gp + m + 12);                 \
        Wn = ld4(w + m + 4);                  \
        hfma4(o, P, Q, Rr, Wc);               \
        Wc = Wn;                              \
        m += 4;                               \
        if (m >= n4) break;                   \
    }
#pragma unroll 1
    for (;;) {
        MP_HSTEP(A, B, C, D)
        MP_HSTEP(B, C, D, A)
        MP_HSTEP(C, D, A, B)
        MP_HSTEP(D, A, B, C)
    }
#undef MP_HSTEP
}

// Vertical over ntaps4 taps (a multiple of 4, zero padded), 8-row register
// ring: tap m uses rows m .. m+3 and loads row m + 7.
__device__ __forceinline__ void v_loop(const float *hp, int stride, const float *w, int ntaps4,
                                       float acc[4][2])
{
#pragma unroll
    for (int o = 0; o < 4; ++o) acc[o][0] = acc[o][1] = 0.f;
    float2 X[8];
#pragma unroll
    for (int j = 0; j < 7; ++j) X[j] = *reinterpret_cast<const float2 *>(hp + j * stride);
    const float *p = hp + 7 * stride;
    int m = 0;
    bool done = false;
#pragma unroll 1
    while (!done) {
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            X[(s + 7) & 7] = *reinterpret_cast<const float2 *>(p);
            p += stride;
            const float wt = w[m + s];
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                acc[o][0] = fmaf(wt, X[(s + o) & 7].x, acc[o][0]);
                acc[o][1] = fmaf(wt, X[(s + o) & 7].y, acc[o][1]);
            }
            if ((s & 3) == 3 && m + s + 1 >= ntaps4) {
                done = true;
                break;
            }
        }
        m += 8;
    }
}

// Issues the TMA loads of input block `blk` of the current item into stage
// `gs % NS` (thread 0 only).
template <int CIN, int RB>
__device__ __forceinline__ void gs_issue(const MPJob &J, const GsGeom &g, float *S, uint64_t *bars,
                                         uint32_t gs, int blk, int gx0, int ybase, int nbx)
{
    const int slot = (int)(gs % (uint32_t)g.NS);
    float *dst = S + slot * g.STG;
    uint64_t *bar = bars + slot;
    mp_mbar_arrive_expect_tx(bar, (uint32_t)(nbx * g.BOXW * RB * 4));
    const int xa = gx0 * CIN;
    const int y = ybase + blk * RB;
    for (int b = 0; b < nbx; ++b) mp_tma_load_2d(dst + b * g.BOXS, &J.tmap, bar, xa + b * g.BOXW, y);
}

// One strip item with compiled bucket radius R (R == 0: loop passes with the
// job's own radius).  `gs` counts the stages this CTA has consumed (it
// selects the stage slot and the mbarrier phase); returns false after a
// timed-out wait (error word set, in-flight copies drained).
template <int CIN, int CMID, int R>
__device__ __noinline__ bool gs_item(const MPJob &J, int lt, const GsGeom &g, unsigned char *base,
                                     uint32_t &gs, bool map_in_global, int *err)
{
    using Cf = GsC<CIN, CMID>;
    constexpr int RB = Cf::RB, NT = Cf::NT, SW = Cf::SW, HW = Cf::HW, LGSW = Cf::LGSW;
    constexpr int LGQPB = GsIn<CIN>::LGQPB;
    constexpr int QPB = GsIn<CIN>::QPB;
    constexpr int RC = R > 0 ? R : 1;                  // compiled radius (unused when R == 0)
    constexpr int NTAPC = 2 * RC + 1;
    constexpr int NT4C = (NTAPC + 3) & ~3;
    uint64_t *bars = reinterpret_cast<uint64_t *>(base);
    float *wv = reinterpret_cast<float *>(base + 64);
    float *wh = wv + 128;
    float *S = reinterpret_cast<float *>(base + g.offS);
    float *G = reinterpret_cast<float *>(base + g.offG);
    float *Hr = reinterpret_cast<float *>(base + g.offH);
    const int tid = threadIdx.x;

    const int sy = lt / J.tiles_x, sx = lt - sy * J.tiles_x;
    const int x0 = sx * SW, y0 = sy * J.th;
    const int H = J.h, W = J.w;
    const int y1 = min(H, y0 + J.th);
    const int r = J.radius;
    const int Rb = R > 0 ? R : r;                      // geometry radius (taps zero padded to it)
    const int R4 = (Rb + 3) & ~3, e = R4 - Rb;
    const int ntv = 2 * Rb + 1;
    const int nth4 = (ntv + e + 3) & ~3;
    const int ntv4 = (ntv + 3) & ~3;
    const int L = (2 * Rb + RB - 1) / RB;
    const int NH = (L + 1) * RB;
    const int nv = (y1 - y0 + RB - 1) / RB;
    const int nb = nv + L;
    const int gx0 = x0 - R4;
    const int ybase = y0 - Rb;
    const int GL = (SW + 2 * R4 + 4 + 15) & ~15;
    const int nq = GL >> 2;
    const int nbx = (GL * CIN + g.BOXW - 1) / g.BOXW;

    __syncthreads();   // the previous item is done with the taps and buffers
    for (int i = tid; i < 128; i += NT) {
        const int k = i - (Rb - r);                    // tap of the job's own filter
        wv[i] = (k >= 0 && k < 2 * r + 1) ? J.wts[k] : 0.f;
        const int kh = k - e;
        wh[i] = (kh >= 0 && kh < 2 * r + 1) ? J.wts[kh] : 0.f;
    }
    if (tid == 0) {
        if (map_in_global) mp_tensormap_acquire(&J.tmap);
        const int pre = min(g.NS - 1, nb);
        for (int k = 0; k < pre; ++k) gs_issue<CIN, RB>(J, g, S, bars, gs + k, k, gx0, ybase, nbx);
    }

    const PwFast pro = mp_pw_fast(J.pro);
    const PwFast epi = mp_pw_fast(J.epi);
    const int npro = J.pro.n;
    const bool grey_pro = npro == 1 && pro.op == MP_OP_RGB2GREY && CIN >= 3;
    // i / nq (P mapping) by multiply-shift: exact for i * nq < 2^20
    const int pdiv = CIN == 3 ? (nq >> 2) : nq;
    const uint32_t pmagic = ((1u << 20) + (uint32_t)pdiv - 1) / (uint32_t)pdiv;
    const int flip = J.flip, wo = J.wo, dp = J.dst_pitch;
    const bool vec = CMID == 1 && !flip && J.vec_out;

    for (int it = 0; it < nb; ++it) {
        const uint32_t gcur = gs + (uint32_t)it;
        if (tid == 0 && it + g.NS - 1 < nb)
            gs_issue<CIN, RB>(J, g, S, bars, gcur + g.NS - 1, it + g.NS - 1, gx0, ybase, nbx);
        const int slot = (int)(gcur % (uint32_t)g.NS);
        const bool ok = mp_mbar_wait_bounded(bars + slot, (gcur / (uint32_t)g.NS) & 1u);

        // ---- P: prologue + de-interleave into G planes, 4 pixels per item
        {
            const float *Sb = S + slot * g.STG;
            const int yb = ybase + it * RB;
            const int total = RB * nq;
            for (int i = tid; i < total; i += NT) {
                int rr, xq;
                if (CIN == 3) {
                    // quarter-warp = 4 quads x 2 rows: conflict-free 48-float box rows
                    const int rest = i >> 3;
                    const int rp = (int)(((uint32_t)rest * pmagic) >> 20);
                    const int xh = rest - rp * pdiv;
                    rr = 2 * rp + ((i >> 2) & 1);
                    xq = 4 * xh + (i & 3);
                } else {
                    rr = (int)(((uint32_t)i * pmagic) >> 20);
                    xq = i - rr * nq;
                }
                const float *sp = Sb + (xq >> LGQPB) * g.BOXS + rr * g.BOXW + (xq & (QPB - 1)) * (4 * CIN);
                float v[4][4];
#pragma unroll
                for (int j = 0; j < CIN; ++j) {
                    const float4 t = ld4(sp + 4 * j);
                    const float tt[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int f = 4 * j + k;
                        v[f / CIN][f % CIN] = tt[k];
                    }
                }
                if (npro) {
                    const int yy = yb + rr;
                    const int px = gx0 + 4 * xq;
                    const bool rowin = (unsigned)yy < (unsigned)H;
                    if (grey_pro) {
#pragma unroll
                        for (int p = 0; p < 4; ++p) {
                            const float gv =
                                fminf(1.0f, 0.2125f * v[p][0] + 0.7154f * v[p][1] + 0.0721f * v[p][2]);
                            v[p][0] = (rowin && (unsigned)(px + p) < (unsigned)W) ? gv : 0.f;
                        }
                    } else {
#pragma unroll
                        for (int p = 0; p < 4; ++p) {
                            if (rowin && (unsigned)(px + p) < (unsigned)W) {
                                mp_pw_apply_f(pro, J.pro, v[p], CIN);
                            } else {
#pragma unroll
                                for (int c = 0; c < CMID; ++c) v[p][c] = 0.f;
                            }
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < CMID; ++c)
                    st4(G + (c * RB + rr) * g.GW + 4 * xq, v[0][c], v[1][c], v[2][c], v[3][c]);
            }
        }
        if (!__syncthreads_and(ok)) {
            if (tid == 0) atomicExch(err, MP_KERR_TIMEOUT);
            // let the copies still in flight land before the CTA exits
            for (int k = it; k < nb && k < it + g.NS; ++k) {
                const uint32_t gk = gs + (uint32_t)k;
                mp_mbar_wait_bounded(bars + gk % (uint32_t)g.NS, (gk / (uint32_t)g.NS) & 1u);
            }
            return false;
        }

        // ---- H: horizontal pass into the ring (rows of this block)
        {
            const int hb = (it * RB) % NH;
            constexpr int NXG = SW / 8;
            constexpr int TOTAL = CMID * RB * NXG;
            float t[NT4C];
            if (R > 0) load_taps<NTAPC>(wv, t);
            for (int i = tid; i < TOTAL; i += NT) {
                const int rr = i & (RB - 1);
                const int xg = (i >> Cf::LGRB) & (NXG - 1);
                const int c = i >> (Cf::LGRB + LGSW - 3);
                float o[8];
                const float *gp = G + (c * RB + rr) * g.GW + 8 * xg;
                if (R > 0) h_item<RC>(gp, t, o);
                else h_loop(gp, wh, nth4, o);
                const int pos = hb + rr;
                float *hp = Hr + (c * g.HR + pos) * HW + 8 * xg;
                st4(hp, o[0], o[1], o[2], o[3]);
                st4(hp + 4, o[4], o[5], o[6], o[7]);
                if (pos < 2 * Rb) {
                    hp += NH * HW;
                    st4(hp, o[0], o[1], o[2], o[3]);
                    st4(hp + 4, o[4], o[5], o[6], o[7]);
                }
            }
        }
        __syncthreads();

        // ---- V: vertical pass for output block it - L, epilogue, store
        if (it >= L) {
            const int v = it - L;
            const int vb = (v * RB) % NH;
            constexpr int NQV = SW / 2;
            constexpr int LGQ = LGSW - 1;
            constexpr int TOTAL = CMID * NQV * (RB / 4);
            float t[NT4C];
            if (R > 0) load_taps<NTAPC>(wv, t);
            for (int i = tid; i < TOTAL; i += NT) {
                const int q = i & (NQV - 1);
                const int grp = (i >> LGQ) & (RB / 4 - 1);
                const int c = i >> (LGQ + Cf::LGRB - 2);
                float acc[4][2];
                const float *hp = Hr + (c * g.HR + vb + 4 * grp) * HW + 2 * q;
                if (R > 0) v_item<RC, HW>(hp, t, acc);
                else v_loop(hp, HW, wv, ntv4, acc);
                const int yb = y0 + v * RB + 4 * grp;
                const int xb = x0 + 2 * q;
                if (xb >= W) continue;
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    const int y = yb + o;
                    if (y >= y1) break;
                    float *drow = J.dst + (size_t)y * dp;
                    const float a0 = mp_pw_chan_f(epi, J.epi, acc[o][0], c, CMID);
                    const float a1 = mp_pw_chan_f(epi, J.epi, acc[o][1], c, CMID);
                    if (vec && xb + 2 <= W) {
                        *reinterpret_cast<float2 *>(drow + xb) = make_float2(a0, a1);
                    } else {
                        drow[(size_t)(flip ? wo - 1 - xb : xb) * CMID + c] = a0;
                        if (xb + 1 < W) drow[(size_t)(flip ? wo - 2 - xb : xb + 1) * CMID + c] = a1;
                    }
                }
            }
        }
    }
    gs += (uint32_t)nb;
    return true;
}

// Runs one item with the compiled bucket of its radius.
// BUCKETS: 0 = loop passes only; 1 = compiled buckets 16 and 24 (smaller
// single-channel radii run on the mp_vh.cuh kernel); 2 = every bucket.
template <int CIN, int CMID, int BUCKETS>
__device__ __forceinline__ bool gs_dispatch(const MPJob &J, int lt, const GsGeom &g, unsigned char *base,
                                            uint32_t &gs, bool map_in_global, int *err)
{
    if constexpr (BUCKETS == 0) return gs_item<CIN, CMID, 0>(J, lt, g, base, gs, map_in_global, err);
    switch (mp_gs_bucket(J.radius)) {
#define MP_GS_CASE(RR) \
    case RR: return gs_item<CIN, CMID, RR>(J, lt, g, base, gs, map_in_global, err);
        MP_GS_CASE(16) MP_GS_CASE(24)
#undef MP_GS_CASE
    default: break;
    }
    if constexpr (BUCKETS == 2) {
        switch (J.radius) {
#define MP_GS_CASE(RR) \
    case RR: return gs_item<CIN, CMID, RR>(J, lt, g, base, gs, map_in_global, err);
            MP_GS_CASE(1) MP_GS_CASE(2) MP_GS_CASE(3) MP_GS_CASE(4) MP_GS_CASE(5) MP_GS_CASE(6)
            MP_GS_CASE(7) MP_GS_CASE(8) MP_GS_CASE(9) MP_GS_CASE(10) MP_GS_CASE(11) MP_GS_CASE(12)
#undef MP_GS_CASE
        default: break;
        }
    }
    return gs_item<CIN, CMID, 0>(J, lt, g, base, gs, map_in_global, err);
}

__device__ __forceinline__ unsigned char *gs_base(unsigned char *smem_raw)
{
    return smem_raw + ((128 - (int)(mp_smem_addr(smem_raw) & 127)) & 127);
}

// Barrier set-up, and zeros in the G and H buffers: the loop passes read a
// few rows and columns past the data they use and multiply some of them by
// zero taps, which must not meet uninitialised (possibly NaN) words.
__device__ __forceinline__ void gs_init(unsigned char *base, const GsGeom &g)
{
    if (threadIdx.x == 0) {
        uint64_t *bars = reinterpret_cast<uint64_t *>(base);
        for (int s = 0; s < g.NS; ++s) mp_mbar_init(bars + s, 1);
        mp_fence_barrier_init();
    }
    float4 *z = reinterpret_cast<float4 *>(base + g.offG);
    const int n4 = (g.total - g.offG) / 16;
    for (int i = threadIdx.x; i < n4; i += blockDim.x) z[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
}

}  // namespace mp_gs

#define MP_GS_KERNELS(NAME, CIN, CMID, BUCKETS)                                                              \
    __global__ void __launch_bounds__(mp_gs_nt(CMID)) NAME##_batch(                                \
        const MPJob *__restrict__ jobs, const int *__restrict__ tile_job, int total,               \
        const __grid_constant__ GsGeom g, int *err)                                                \
    {                                                                                              \
        extern __shared__ unsigned char mp_gs_smem[];                                              \
        unsigned char *base = mp_gs::gs_base(mp_gs_smem);                                                 \
        mp_gs::gs_init(base, g);                                                                  \
        uint32_t gs = 0;                                                                           \
        for (int t = blockIdx.x; t < total; t += gridDim.x) {                                      \
            const MPJob &J = jobs[__ldg(tile_job + t)];                                            \
            if (!mp_gs::gs_dispatch<CIN, CMID, BUCKETS>(J, t - J.tile0, g, base, gs, true, err)) return;           \
        }                                                                                          \
    }                                                                                              \
    __global__ void __launch_bounds__(mp_gs_nt(CMID))                                              \
        NAME##_single(const __grid_constant__ MPJob job, const __grid_constant__ GsGeom g, int *err) \
    {                                                                                              \
        extern __shared__ unsigned char mp_gs_smem[];                                              \
        unsigned char *base = mp_gs::gs_base(mp_gs_smem);                                                 \
        mp_gs::gs_init(base, g);                                                                  \
        uint32_t gs = 0;                                                                           \
        for (int t = blockIdx.x; t < job.ntiles; t += gridDim.x)                                   \
            if (!mp_gs::gs_dispatch<CIN, CMID, BUCKETS>(job, t, g, base, gs, false, err)) return;                  \
    }

