// mp_vh.cuh -- the separable gaussian as one streaming kernel (sm_103a):
// vertical pass in registers, horizontal pass through a small shared-memory
// tile.
//
// Same operator as the other gaussian kernels (zero-padded separable
// correlation with normalised exp(-k^2 / 2 sigma^2) taps, radius
// ceil(3 sigma); the reference's weights and padding are
// src/millipyde_image.cpp:745-756 and :170-172, :218-221).  Two families:
//   CM = 1   segments whose channel count after the prologue is 1: an
//            rgb2grey prologue on 3- or 4-channel sources, or a 1-channel
//            source with a pointwise prologue.  A column is a pixel.
//   CM = C   channel-preserving segments on C = 3 or 4 interleaved channels
//            (per-channel prologue / epilogue, no rgb2grey).  A column is
//            one float of the interleaved row: the vertical pass does not
//            care which channel a float belongs to, and the horizontal taps
//            step by C floats.
//
// A work item is a STRIP of at most 2*NT - 2*R4 output columns (R4 = R*CM
// rounded up to 4; the width is fitted to each image) by RS output rows.
// Each thread owns two adjacent columns of the strip plus its halo and
// walks down them:
//   load   one thread copies the source rows of the strip, 8 at a time, by
//          TMA (one box of 64 pixels per warp) into a double-buffered
//          staging area, the next 8 rows in flight while the current ones
//          are filtered; boxes that leave the image arrive as zeros, and
//          pixels outside the image read as 0 after the prologue.
//   V      a register window of 8 + 2R rows of (prologued) column pairs; each
//          step produces 8 vertical outputs per column with packed f32x2
//          FMAs, then slides the window by 8 rows.
//   H      the 8 vertical rows go to a double-buffered shared tile, rows 2p
//          and 2p + 1 interleaved per column; after one barrier every thread
//          computes 8 consecutive horizontal outputs of two rows at once
//          (each tap one f32x2 FMA on a (row 2p, row 2p + 1) pair) and
//          applies the epilogue and fliplr map.
// The radius is a compile-time parameter (one instance per radius 1..12).
#pragma once
#include "mp_internal.cuh"

#define MP_VH_NT 128       // threads of a CTA (2 columns each)
#define MP_VH_NT_BIG 256   // threads of the radius-bucket kernels: wider strips, the halo a smaller share
#define MP_VH_VR 8
// Largest radius at which the channel-preserving family pairs output rows
// in the horizontal pass (one f32x2 FMA per tap for two rows).  Measured on
// interleaved RGB: radii 1..4 about 5 % faster paired; 5..8 spill at the
// 128-register budget of their kernel and 9..12 ran 7 % slower.
#ifndef MP_VH_PAIR_RMAX
#define MP_VH_PAIR_RMAX 4
#endif

namespace mp_vh {

__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

// d = a * b + c on float pairs (one f32x2 instruction).
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;"
        : "=l"(d)
        : "l"(*reinterpret_cast<unsigned long long *>(&a)), "l"(*reinterpret_cast<unsigned long long *>(&b)),
          "l"(*reinterpret_cast<unsigned long long *>(&c)));
    return *reinterpret_cast<float2 *>(&d);
}

// d = a + b on float pairs.
__device__ __forceinline__ float2 add2(float2 a, float2 b)
{
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;"
        : "=l"(d)
        : "l"(*reinterpret_cast<unsigned long long *>(&a)), "l"(*reinterpret_cast<unsigned long long *>(&b)));
    return *reinterpret_cast<float2 *>(&d);
}

// Prologue of the two staged pixels -> one value each; in0 / in1 say
// whether each pixel lies inside the image (zero otherwise, after the
// prologue: the zero padding of the blur).
template <int CIN>
__device__ __forceinline__ float2 prologue(const float *slot, bool in0, bool in1, bool grey_only, const PwFast &pro,
                                           const PwList &L)
{
    float r[2 * CIN];
    if (CIN == 4) {
        const float4 a = ld4(slot), b = ld4(slot + 4);
        r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w;
        r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
    } else {
#pragma unroll
        for (int k = 0; k < CIN; ++k) {
            const float2 t = *reinterpret_cast<const float2 *>(slot + 2 * k);
            r[2 * k] = t.x;
            r[2 * k + 1] = t.y;
        }
    }
    float2 o;
    if (CIN >= 3 && grey_only) {
        o.x = fminf(1.0f, 0.2125f * r[0] + 0.7154f * r[1] + 0.0721f * r[2]);
        o.y = fminf(1.0f, 0.2125f * r[CIN] + 0.7154f * r[CIN + 1] + 0.0721f * r[CIN + 2]);
    } else {
        float a[4] = {0.f, 0.f, 0.f, 0.f}, b[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int k = 0; k < CIN; ++k) {
            a[k] = r[k];
            b[k] = r[CIN + k];
        }
        mp_pw_apply_f(pro, L, a, CIN);
        mp_pw_apply_f(pro, L, b, CIN);
        o.x = a[0];
        o.y = b[0];
    }
    o.x = in0 ? o.x : 0.f;
    o.y = in1 ? o.y : 0.f;
    return o;
}

// Shared memory of one CTA (floats): 2 mbarriers + taps (64 floats), two
// horizontal tiles [2][VR][VW], two staging buffers [2][NW][VR][64*PX]
// (PX = floats staged per column: CIN when CM = 1, else 1), then the 64
// horizontal taps of the dot mode.
__host__ __device__ constexpr int mp_vh_smem_floats(int cin, int cm, int nt = MP_VH_NT)
{
    return 64 + 64 + 2 * MP_VH_VR * (2 * nt + 4) + 2 * MP_VH_VR * 2 * nt * (cm == 1 ? cin : 1) + 64;
}

// Channel of interleaved float column f (f may be negative: halo columns).
template <int CM>
__device__ __forceinline__ int chan_of(int f)
{
    const int c = f % CM;
    return c < 0 ? c + CM : c;
}

// One strip item with compiled radius R.  The strip is J.tw output columns
// wide (a multiple of 8, at most 2*NT - 2*R4); window rows are counted from
// source row y0 - R8 (R8 = R rounded up to 4) so that every step of VR rows
// is exactly one staged group.
// Radii above MP_VH_RMAX are buckets: a job of radius r <= R runs with its
// taps centred in 2R + 1 (zeros outside), the vertical pass adds the two
// window rows of each symmetric tap pair before multiplying (R + 1 tap
// registers instead of 2R + 1) and the horizontal pass consumes the tile row
// in order.
// DOT: the d sigma mode of the gaussian's adjoint.  The horizontal pass
// uses J.wts_h (the vertical pass J.wts), nothing is stored, and the sum of
// output * J.aux (the output-space gradient) over the item is added to
// J.acc[0] in FP64 (one atomic per warp and item).
template <int CIN, int CM, int R, bool DOT = false, int NT = MP_VH_NT>
__device__ __noinline__ void vh_item(const MPJob &J, int lt, float *smem, uint32_t &gcount, int *err)
{
    constexpr bool BIG = R > MP_VH_RMAX;
    constexpr int VR = MP_VH_VR, VW = 2 * NT + 4, NW = NT / 32;
    constexpr int NTAP = 2 * R + 1, RC = R * CM, R4 = (RC + 3) & ~3, E = R4 - RC;
    constexpr int NW2 = BIG ? R + 1 : NTAP;               // tap registers
    // the plain one-channel family computes two output rows per
    // horizontal work item as packed pairs, and so does the channel-
    // preserving family up to radius MP_VH_PAIR_RMAX; the radius buckets do
    // not (256 threads, 1 CTA per SM: paired measured slower, 97.7 against
    // 87.5 ms for a training step with two radius-24 blurs per 8192x8192 RGB
    // image)
    constexpr bool PAIR = !BIG && !DOT && (CM == 1 || R <= MP_VH_PAIR_RMAX);
    constexpr int R8 = (R + 3) & ~3;                      // window row padding (2*R8 is a multiple of 8)
    constexpr int D = R8 - R;                             // tap offset inside the window
    constexpr int NWIN = VR + 2 * R8;
    constexpr int NPRE = 2 * R8 / VR;                     // groups holding the window head
    constexpr int NLD = (E + 8 + 2 * RC + 3) / 4;
    constexpr int PX = CM == 1 ? CIN : 1;                 // staged floats per column
    constexpr int BOXW = 64 * PX;                         // staged floats per warp and row
    constexpr int GF = NW * VR * BOXW;                    // staged floats per group
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    float *taps = smem + 64;
    float *tile = smem + 128;
    float *stg = tile + 2 * VR * VW;                      // [2][NW][VR][BOXW]
    float *taps_h = stg + 2 * GF;                         // DOT: horizontal taps

    const int sy = lt / J.tiles_x, sx = lt - sy * J.tiles_x;
    const int H = J.h, W = J.w * CM;                      // W in columns
    const int swo = J.tw, ng = swo >> 3;
    const int x0 = sx * swo, y0 = sy * J.th;
    const int y1 = min(H, y0 + J.th);
    const int nsteps = (y1 - y0 + VR - 1) / VR;
    const int xv = x0 - R4 + 2 * tid;                     // this thread's first column
    const bool in0 = xv >= 0 && xv < W, in1 = xv + 1 >= 0 && xv + 1 < W;
    const int ch0 = chan_of<CM>(xv), ch1 = chan_of<CM>(xv + 1);
    const int ybase = y0 - R8;                            // source row of window row 0

    __syncthreads();   // the previous item is done with the taps, tiles and staging
    if constexpr (BIG) {
        const int sh = R - J.radius;                      // bucket shift of the job's taps
        if (tid < 64) taps[tid] = (tid >= sh && tid < NTAP - sh) ? J.wts[tid - sh] : 0.f;
    } else {
        if (tid < 64) taps[tid] = tid < NTAP ? J.wts[tid] : 0.f;
    }
    if constexpr (DOT) {
        if (tid < 64) taps_h[tid] = tid < NTAP ? J.wts_h[tid] : 0.f;
    }
    const PwFast pro = mp_pw_fast(J.pro);
    const bool grey_only = J.pro.n == 1 && pro.op == MP_OP_RGB2GREY;
    const PwFast epi = mp_pw_fast(J.epi);
    PwRegs pro3, epi3;   // the channel-preserving family's lists in registers
    if constexpr (CM > 1) {
        pro3 = mp_pw_regs(J.pro);
        epi3 = mp_pw_regs(J.epi);
    }
    const int flip = J.flip, wo = J.wo, dp = J.dst_pitch;
    const bool vec = !flip && J.vec_out;
    float *const dst = J.dst;
    const uint32_t g0 = gcount;                           // CTA-wide group counter at item start
    const int ngroups = NPRE + nsteps;

    // thread 0: TMA of window group g (rows [VR g, VR g + VR)) into buffer (g0+g) & 1
    auto issue = [&](int g) {
        const uint32_t G = g0 + (uint32_t)g;
        uint64_t *bar = bars + (G & 1u);
        float *b = stg + (G & 1u) * GF;
        mp_mbar_arrive_expect_tx(bar, (uint32_t)(GF * 4));
        for (int w = 0; w < NW; ++w)
            mp_tma_load_2d(b + w * VR * BOXW, &J.tmap, bar, (x0 - R4 + 64 * w) * PX, ybase + VR * g);
    };
    // all threads: wait for group g; false after a timeout (error word set)
    auto wait = [&](int g) -> bool {
        const uint32_t G = g0 + (uint32_t)g;
        const bool ok = mp_mbar_wait_bounded(bars + (G & 1u), (G >> 1) & 1u);
        if (__syncthreads_and(ok)) return true;
        if (tid == 0) atomicExch(err, MP_KERR_TIMEOUT);
        return false;
    };
    // prologue of the VR rows of group g for this thread's two pixels, into
    // win[w0 .. w0 + VR): the prologue kind is decided once per group
    auto group_values = [&](int g, float2 *wdst) {
        const uint32_t G = g0 + (uint32_t)g;
        const float *slot = stg + (G & 1u) * GF + warp * VR * BOXW + lane * 2 * PX;
        const int yr = ybase + VR * g;
        if constexpr (CM > 1) {
            // interleaved floats: per-channel prologue on each column
            if (J.pro.n) {
                float v[2 * VR];
                int chv[2 * VR];
#pragma unroll
                for (int j = 0; j < VR; ++j) {
                    const float2 t = *reinterpret_cast<const float2 *>(slot + j * BOXW);
                    v[2 * j] = t.x;
                    v[2 * j + 1] = t.y;
                    chv[2 * j] = ch0;
                    chv[2 * j + 1] = ch1;
                }
                mp_pw_chan_n<2 * VR>(pro3, J.pro, v, chv, CM);
#pragma unroll
                for (int j = 0; j < VR; ++j) {
                    const bool rin = (unsigned)(yr + j) < (unsigned)H;
                    wdst[j] = make_float2(in0 && rin ? v[2 * j] : 0.f, in1 && rin ? v[2 * j + 1] : 0.f);
                }
            } else {
                // no prologue: the copy's zero fill already pads the image
#pragma unroll
                for (int j = 0; j < VR; ++j) wdst[j] = *reinterpret_cast<const float2 *>(slot + j * BOXW);
            }
        } else if (CIN >= 3 && grey_only) {
#pragma unroll
            for (int j = 0; j < VR; ++j) {
                const bool rin = (unsigned)(yr + j) < (unsigned)H;
                wdst[j] = prologue<CIN>(slot + j * BOXW, in0 && rin, in1 && rin, true, pro, J.pro);
            }
        } else {
#pragma unroll
            for (int j = 0; j < VR; ++j) {
                const bool rin = (unsigned)(yr + j) < (unsigned)H;
                wdst[j] = prologue<CIN>(slot + j * BOXW, in0 && rin, in1 && rin, false, pro, J.pro);
            }
        }
    };

    if (tid == 0) {
        mp_tensormap_acquire(&J.tmap);
        issue(0);
    }
    __syncthreads();
    float2 w2[NW2];
#pragma unroll
    for (int m = 0; m < NW2; ++m) w2[m] = make_float2(taps[m], taps[m]);
    // tap m of 2R + 1 (symmetric storage for the buckets)
    auto tap = [&](int m) -> float { return BIG ? w2[m <= R ? m : 2 * R - m].x : w2[m].x; };
    float hw[DOT ? NTAP : 1];
    if constexpr (DOT) {
#pragma unroll
        for (int m = 0; m < NTAP; ++m) hw[m] = taps_h[m];
    }
    // horizontal tap m
    auto htap = [&](int m) -> float {
        if constexpr (DOT) return hw[m];
        else return tap(m);
    };
    float dacc = 0.f;   // DOT: this thread's share of sum(out * aux)
    const bool aux_vec = DOT && ((uintptr_t)J.aux & 15) == 0 && (J.aux_pitch & 3) == 0;

    float2 win[NWIN];
    bool alive = true;
    // window head: rows 0 .. 2*R8-1 (groups 0 .. NPRE-1).  The head values
    // stay in registers until the first vertical step, but the buffer they
    // came from receives group g + 2 by TMA right after the next barrier: a
    // shared-memory load still queued behind this thread's earlier stores
    // would then return the newer rows.  The barrier's predicate depends on
    // every loaded value, so each thread's loads of group g have completed
    // before it arrives (the predicate itself is never true for finite data).
#pragma unroll
    for (int g = 0; g < NPRE; ++g) {
        if (tid == 0) issue(g + 1);            // its buffer was read in iteration g - 1
        alive = alive && wait(g);
        group_values(g, win + VR * g);
        float chk = 0.f;
#pragma unroll
        for (int j = 0; j < VR; ++j) chk += win[VR * g + j].x + win[VR * g + j].y;
        __syncthreads_or(chk == 3.0e38f);
    }

    for (int s = 0; s <= nsteps; ++s) {
        if (s < nsteps && alive) {
            // ---- V: group NPRE + s = window rows 2*R8 .. 2*R8 + VR - 1
            const int gB = NPRE + s;
            if (tid == 0 && gB + 1 < ngroups) issue(gB + 1);   // buffer of group gB - 1, read last step
            alive = wait(gB);
            group_values(gB, win + 2 * R8);
            // PAIR: rows 2p and 2p + 1 interleaved per column (one float4 per
            // row pair holds the thread's two columns of both rows); else
            // row by row
            float *tb = tile + (s & 1) * (VR * VW) + (PAIR ? 4 : 2) * tid;
            float2 prev = make_float2(0.f, 0.f);
#pragma unroll
            for (int o = 0; o < VR; ++o) {
                float2 a = make_float2(0.f, 0.f);
                if constexpr (BIG) {
                    a = fma2(w2[R], win[o + D + R], a);
#pragma unroll
                    for (int k = 0; k < R; ++k) a = fma2(w2[k], add2(win[o + D + k], win[o + D + 2 * R - k]), a);
                } else {
#pragma unroll
                    for (int k = 0; k < NTAP; ++k) a = fma2(w2[k], win[o + D + k], a);
                }
                if constexpr (PAIR) {
                    if (o & 1)
                        *reinterpret_cast<float4 *>(tb + (o >> 1) * (2 * VW)) = make_float4(prev.x, a.x, prev.y, a.y);
                    else
                        prev = a;
                } else {
                    *reinterpret_cast<float2 *>(tb + o * VW) = a;
                }
            }
#pragma unroll
            for (int k = 0; k < 2 * R8; ++k) win[k] = win[k + VR];
        }
        if (s >= 1 && alive) {
        if constexpr (PAIR) {
            // ---- H: output rows of step s-1 from its shared tile, two rows
            // per work item as packed pairs (one f32x2 FMA per tap for both)
            const int sb = s - 1;
            const float *tr = tile + (sb & 1) * (VR * VW);
            for (int i = tid; i < (VR / 2) * ng; i += NT) {
                const int rp = i & (VR / 2 - 1), g = i >> 2;
                const int ya = y0 + VR * sb + 2 * rp;
                const int xo0 = x0 + 8 * g;
                if (ya >= y1 || xo0 >= W) continue;
                const float *gp = tr + rp * (2 * VW) + 16 * g;   // column pairs from 8g on
                float2 o2[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) o2[k] = make_float2(0.f, 0.f);
                // consume the column pairs in order so that only the 8 sums
                // stay live; taps CM columns apart (tap order per output)
#pragma unroll
                for (int q = 0; q < 2 * NLD; ++q) {
                    const float4 v = ld4(gp + 4 * q);
                    const float2 pc[2] = {make_float2(v.x, v.y), make_float2(v.z, v.w)};
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
#pragma unroll
                        for (int k = 0; k < 8; ++k) {
                            const int t = 2 * q + u - E - k;   // = m * CM for tap m
                            if (t >= 0 && t % CM == 0 && t / CM < NTAP) {
                                if constexpr (DOT) {
                                    o2[k].x = fmaf(hw[t / CM], pc[u].x, o2[k].x);
                                    o2[k].y = fmaf(hw[t / CM], pc[u].y, o2[k].y);
                                } else {
                                    const int m = t / CM;
                                    o2[k] = fma2(w2[BIG ? (m <= R ? m : 2 * R - m) : m], pc[u], o2[k]);
                                }
                            }
                        }
                    }
                }
                // epilogue / store (or the dot product) of one output row
                auto emit = [&](float (&o)[8], int y) {
                    if constexpr (DOT) {
                        const float *arow = J.aux + (size_t)y * J.aux_pitch;
                        if (aux_vec && xo0 + 8 <= W) {
                            const float4 p = ld4(arow + xo0), q = ld4(arow + xo0 + 4);
                            dacc = fmaf(o[0], p.x, dacc);
                            dacc = fmaf(o[1], p.y, dacc);
                            dacc = fmaf(o[2], p.z, dacc);
                            dacc = fmaf(o[3], p.w, dacc);
                            dacc = fmaf(o[4], q.x, dacc);
                            dacc = fmaf(o[5], q.y, dacc);
                            dacc = fmaf(o[6], q.z, dacc);
                            dacc = fmaf(o[7], q.w, dacc);
                        } else {
#pragma unroll
                            for (int k = 0; k < 8; ++k)
                                if (xo0 + k < W) dacc = fmaf(o[k], arow[xo0 + k], dacc);
                        }
                        return;
                    }
                    if (epi.n) {
                        if constexpr (CM == 1) {
#pragma unroll
                            for (int k = 0; k < 8; ++k) o[k] = mp_pw_chan_f(epi, J.epi, o[k], 0, 1);
                        } else {
                            const int cb = xo0 % CM;
                            int chv[8];
#pragma unroll
                            for (int k = 0; k < 8; ++k) chv[k] = (cb + k) % CM;
                            mp_pw_chan_n<8>(epi3, J.epi, o, chv, CM);
                        }
                    }
                    float *drow = dst + (size_t)y * dp;
                    if (vec && xo0 + 8 <= W) {
                        *reinterpret_cast<float4 *>(drow + xo0) = make_float4(o[0], o[1], o[2], o[3]);
                        *reinterpret_cast<float4 *>(drow + xo0 + 4) = make_float4(o[4], o[5], o[6], o[7]);
                    } else if constexpr (CM == 1) {
#pragma unroll
                        for (int k = 0; k < 8; ++k)
                            if (xo0 + k < W) drow[flip ? wo - 1 - (xo0 + k) : xo0 + k] = o[k];
                    } else if (CM == 4 && flip && J.vec_out && xo0 + 8 <= W) {
                        // two whole pixels, mirrored: one float4 each
                        const int px = xo0 >> 2;
                        *reinterpret_cast<float4 *>(drow + (wo - 1 - px) * 4) = make_float4(o[0], o[1], o[2], o[3]);
                        *reinterpret_cast<float4 *>(drow + (wo - 2 - px) * 4) = make_float4(o[4], o[5], o[6], o[7]);
                    } else {
                        // fliplr mirrors pixels and keeps the channel order
#pragma unroll
                        for (int k = 0; k < 8; ++k) {
                            const int f = xo0 + k;
                            if (f < W) {
                                const int px = f / CM, c = f - px * CM;
                                drow[flip ? (wo - 1 - px) * CM + c : f] = o[k];
                            }
                        }
                    }
                };
                float oa[8], ob[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    oa[k] = o2[k].x;
                    ob[k] = o2[k].y;
                }
                emit(oa, ya);
                if (ya + 1 < y1) emit(ob, ya + 1);
            }
        } else {
            // ---- H: output rows of step s-1 from its shared tile
            const int sb = s - 1;
            const float *tr = tile + (sb & 1) * (VR * VW);
            for (int i = tid; i < VR * ng; i += NT) {
                const int rr = i & (VR - 1), g = i >> 3;
                const int y = y0 + VR * sb + rr;
                const int xo0 = x0 + 8 * g;
                if (y >= y1 || xo0 >= W) continue;
                const float *gp = tr + rr * VW + 8 * g;
                float o[8];
                if constexpr (CM == 1 && !BIG) {
                    float x[4 * NLD];
#pragma unroll
                    for (int q = 0; q < NLD; ++q) {
                        const float4 v = ld4(gp + 4 * q);
                        x[4 * q] = v.x;
                        x[4 * q + 1] = v.y;
                        x[4 * q + 2] = v.z;
                        x[4 * q + 3] = v.w;
                    }
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        float a0 = 0.f, a1 = 0.f;
#pragma unroll
                        for (int m = 0; m < NTAP; ++m) {
                            if (m & 1) a1 = fmaf(htap(m), x[E + k + m], a1);
                            else a0 = fmaf(htap(m), x[E + k + m], a0);
                        }
                        o[k] = a0 + a1;
                    }
                } else if constexpr (!DOT) {
                    // taps CM floats apart: consume the tile row in order so
                    // that only the 8 sums stay live.  Outputs 2j and 2j + 1
                    // use the same tap at positions p and p + 1: where p is
                    // even the two operands are one aligned register pair of
                    // the float4 and take one f32x2 FMA, else two scalar
                    // FMAs (an operand that opens the next float4 is added
                    // there).  Each output still sums its taps in position
                    // order.
                    float2 o2[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j) o2[j] = make_float2(0.f, 0.f);
#pragma unroll
                    for (int q = 0; q < NLD; ++q) {
                        const float4 v = ld4(gp + 4 * q);
                        const float e4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            // output 2j + 1 at position 4q, its tap found at 4q - 1 for output 2j
                            const int t = 4 * q - 1 - E - 2 * j;
                            if (q > 0 && t >= 0 && t % CM == 0 && t / CM < NTAP)
                                o2[j].y = fmaf(htap(t / CM), e4[0], o2[j].y);
                        }
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
#pragma unroll
                            for (int j = 0; j < 4; ++j) {
                                const int t = 4 * q + u - E - 2 * j;   // = m * CM for tap m of output 2j
                                if (t >= 0 && t % CM == 0 && t / CM < NTAP) {
                                    const int m = t / CM;
                                    if (u % 2 == 0) {
                                        o2[j] = fma2(w2[BIG ? (m <= R ? m : 2 * R - m) : m],
                                                     make_float2(e4[u], e4[u + 1]), o2[j]);
                                    } else {
                                        o2[j].x = fmaf(htap(m), e4[u], o2[j].x);
                                        if (u == 1) o2[j].y = fmaf(htap(m), e4[2], o2[j].y);
                                    }
                                }
                            }
                        }
                    }
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        o[2 * j] = o2[j].x;
                        o[2 * j + 1] = o2[j].y;
                    }
                } else {
                    // taps CM floats apart: consume the tile row in order so
                    // that only the 8 sums stay live (tap order per output)
#pragma unroll
                    for (int k = 0; k < 8; ++k) o[k] = 0.f;
#pragma unroll
                    for (int q = 0; q < NLD; ++q) {
                        const float4 v = ld4(gp + 4 * q);
                        const float e4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
#pragma unroll
                            for (int k = 0; k < 8; ++k) {
                                const int t = 4 * q + u - E - k;   // = m * CM for tap m
                                if (t >= 0 && t % CM == 0 && t / CM < NTAP) o[k] = fmaf(htap(t / CM), e4[u], o[k]);
                            }
                        }
                    }
                }
                if constexpr (DOT) {
                    const float *arow = J.aux + (size_t)y * J.aux_pitch;
                    if (aux_vec && xo0 + 8 <= W) {
                        const float4 p = ld4(arow + xo0), q = ld4(arow + xo0 + 4);
                        dacc = fmaf(o[0], p.x, dacc);
                        dacc = fmaf(o[1], p.y, dacc);
                        dacc = fmaf(o[2], p.z, dacc);
                        dacc = fmaf(o[3], p.w, dacc);
                        dacc = fmaf(o[4], q.x, dacc);
                        dacc = fmaf(o[5], q.y, dacc);
                        dacc = fmaf(o[6], q.z, dacc);
                        dacc = fmaf(o[7], q.w, dacc);
                    } else {
#pragma unroll
                        for (int k = 0; k < 8; ++k)
                            if (xo0 + k < W) dacc = fmaf(o[k], arow[xo0 + k], dacc);
                    }
                    continue;
                }
                if (epi.n) {
                    if constexpr (CM == 1) {
#pragma unroll
                        for (int k = 0; k < 8; ++k) o[k] = mp_pw_chan_f(epi, J.epi, o[k], 0, 1);
                    } else {
                        const int cb = xo0 % CM;
                        int chv[8];
#pragma unroll
                        for (int k = 0; k < 8; ++k) chv[k] = (cb + k) % CM;
                        mp_pw_chan_n<8>(epi3, J.epi, o, chv, CM);
                    }
                }
                float *drow = dst + (size_t)y * dp;
                if (vec && xo0 + 8 <= W) {
                    *reinterpret_cast<float4 *>(drow + xo0) = make_float4(o[0], o[1], o[2], o[3]);
                    *reinterpret_cast<float4 *>(drow + xo0 + 4) = make_float4(o[4], o[5], o[6], o[7]);
                } else if constexpr (CM == 1) {
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        if (xo0 + k < W) drow[flip ? wo - 1 - (xo0 + k) : xo0 + k] = o[k];
                } else if (CM == 4 && flip && J.vec_out && xo0 + 8 <= W) {
                    // two whole pixels, mirrored: one float4 each
                    const int px = xo0 >> 2;
                    *reinterpret_cast<float4 *>(drow + (wo - 1 - px) * 4) = make_float4(o[0], o[1], o[2], o[3]);
                    *reinterpret_cast<float4 *>(drow + (wo - 2 - px) * 4) = make_float4(o[4], o[5], o[6], o[7]);
                } else {
                    // fliplr mirrors pixels and keeps the channel order
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const int f = xo0 + k;
                        if (f < W) {
                            const int px = f / CM, c = f - px * CM;
                            drow[flip ? (wo - 1 - px) * CM + c : f] = o[k];
                        }
                    }
                }
            }
        }
        }
        __syncthreads();
    }
    // after a timeout: let the copies still in flight (the last groups
    // issued, one per buffer) land before the buffers are reused
    if (!alive) {
        for (int g = ngroups - 2; g < ngroups; ++g) {
            if (g < 0) continue;
            const uint32_t G = g0 + (uint32_t)g;
            mp_mbar_wait_bounded(bars + (G & 1u), (G >> 1) & 1u);
        }
    }
    gcount = g0 + (uint32_t)ngroups;
    if constexpr (DOT) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dacc += __shfl_down_sync(0xffffffffu, dacc, o);
        if (lane == 0 && alive) atomicAdd(J.acc, (double)dacc);
    }
}

template <int CIN, int CM>
__device__ __forceinline__ void vh_dispatch(const MPJob &J, int lt, float *smem, uint32_t &gc, int *err)
{
    switch (J.radius) {
#define MP_VH_CASE(RR) \
    case RR: vh_item<CIN, CM, RR>(J, lt, smem, gc, err); break;
        MP_VH_CASE(1) MP_VH_CASE(2) MP_VH_CASE(3) MP_VH_CASE(4) MP_VH_CASE(5) MP_VH_CASE(6)
        MP_VH_CASE(7) MP_VH_CASE(8) MP_VH_CASE(9) MP_VH_CASE(10) MP_VH_CASE(11) MP_VH_CASE(12)
#undef MP_VH_CASE
    default: break;   // the planner never sends other radii here
    }
}

// Radius groups of the exact-radius kernels, compiled as separate kernels
// so that each is allocated registers for its own radii (smaller radii:
// smaller windows, more resident CTAs per SM): 1..4, 5..8, 9..12.
template <int CIN, int CM>
__device__ __forceinline__ void vh_dispatch_lo(const MPJob &J, int lt, float *smem, uint32_t &gc, int *err)
{
    switch (J.radius) {
#define MP_VH_CASE(RR) \
    case RR: vh_item<CIN, CM, RR>(J, lt, smem, gc, err); break;
        MP_VH_CASE(1) MP_VH_CASE(2) MP_VH_CASE(3) MP_VH_CASE(4)
#undef MP_VH_CASE
    default: break;
    }
}

template <int CIN, int CM>
__device__ __forceinline__ void vh_dispatch_mid(const MPJob &J, int lt, float *smem, uint32_t &gc, int *err)
{
    switch (J.radius) {
#define MP_VH_CASE(RR) \
    case RR: vh_item<CIN, CM, RR>(J, lt, smem, gc, err); break;
        MP_VH_CASE(5) MP_VH_CASE(6) MP_VH_CASE(7) MP_VH_CASE(8)
#undef MP_VH_CASE
    default: break;
    }
}

template <int CIN, int CM>
__device__ __forceinline__ void vh_dispatch_hi(const MPJob &J, int lt, float *smem, uint32_t &gc, int *err)
{
    switch (J.radius) {
#define MP_VH_CASE(RR) \
    case RR: vh_item<CIN, CM, RR>(J, lt, smem, gc, err); break;
        MP_VH_CASE(9) MP_VH_CASE(10) MP_VH_CASE(11) MP_VH_CASE(12)
#undef MP_VH_CASE
    default: break;
    }
}

// The d sigma dot mode, radii 1..MP_VH_RMAX.
template <int CIN, int CM>
__device__ __forceinline__ void vh_dispatch_dot(const MPJob &J, int lt, float *smem, uint32_t &gc, int *err)
{
    switch (J.radius) {
#define MP_VH_CASE(RR) \
    case RR: vh_item<CIN, CM, RR, true>(J, lt, smem, gc, err); break;
        MP_VH_CASE(1) MP_VH_CASE(2) MP_VH_CASE(3) MP_VH_CASE(4) MP_VH_CASE(5) MP_VH_CASE(6)
        MP_VH_CASE(7) MP_VH_CASE(8) MP_VH_CASE(9) MP_VH_CASE(10) MP_VH_CASE(11) MP_VH_CASE(12)
#undef MP_VH_CASE
    default: break;
    }
}

// Radii above MP_VH_RMAX, rounded up to a bucket.
template <int CIN, int CM>
__device__ __forceinline__ void vh_dispatch_big(const MPJob &J, int lt, float *smem, uint32_t &gc, int *err)
{
    if (J.radius <= 16) vh_item<CIN, CM, 16, false, MP_VH_NT_BIG>(J, lt, smem, gc, err);
    else if (J.radius <= 20) vh_item<CIN, CM, 20, false, MP_VH_NT_BIG>(J, lt, smem, gc, err);
    else if (J.radius <= MP_VH_RBIG) vh_item<CIN, CM, MP_VH_RBIG, false, MP_VH_NT_BIG>(J, lt, smem, gc, err);
}

__device__ __forceinline__ float *vh_base(float4 *raw)
{
    unsigned char *p = reinterpret_cast<unsigned char *>(raw);
    return reinterpret_cast<float *>(p + ((128 - (int)(mp_smem_addr(p) & 127)) & 127));
}

__device__ __forceinline__ void vh_init(float *smem)
{
    if (threadIdx.x == 0) {
        uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
        mp_mbar_init(bars, 1);
        mp_mbar_init(bars + 1, 1);
        mp_fence_barrier_init();
    }
    __syncthreads();
}

}  // namespace mp_vh

// Persistent kernels: CTA b takes strip items b, b + grid, ...
#define MP_VH_KERNELS_X(NAME, CIN, CM, DISPATCH, MINB, NTH)                                                                 \
    __global__ void __launch_bounds__(NTH, MINB) NAME##_batch(                                    \
        const MPJob *__restrict__ jobs, const int *__restrict__ tile_job, int total, int *err,      \
        int *counter)                                                                               \
    {                                                                                               \
        extern __shared__ float4 mp_vh_dsmem4[];                                                    \
        __shared__ int next_item;                                                                   \
        float *smem = mp_vh::vh_base(mp_vh_dsmem4);                                                 \
        mp_vh::vh_init(smem);                                                                       \
        uint32_t gc = 0;                                                                            \
        /* first item by CTA index, the rest from the launch's counter */                          \
        for (int t = blockIdx.x; t < total;) {                                                      \
            const MPJob &J = jobs[__ldg(tile_job + t)];                                             \
            mp_vh::DISPATCH<CIN, CM>(J, t - J.tile0, smem, gc, err);                                 \
            __syncthreads(); /* every thread has read next_item */                                  \
            if (threadIdx.x == 0) next_item = (int)gridDim.x + atomicAdd(counter, 1);              \
            __syncthreads();                                                                        \
            t = next_item;                                                                          \
        }                                                                                           \
    }                                                                                               \
    __global__ void __launch_bounds__(NTH, MINB)                                                  \
        NAME##_single(const __grid_constant__ MPJob job, int *err)                                  \
    {                                                                                               \
        extern __shared__ float4 mp_vh_dsmem4[];                                                    \
        float *smem = mp_vh::vh_base(mp_vh_dsmem4);                                                 \
        mp_vh::vh_init(smem);                                                                       \
        uint32_t gc = 0;                                                                            \
        for (int t = blockIdx.x; t < job.ntiles; t += gridDim.x)                                    \
            mp_vh::DISPATCH<CIN, CM>(job, t, smem, gc, err);                                         \
    }

// Radii 1..MP_VH_RMAX and the d sigma dot mode (128 threads, 3 CTAs per SM;
// the dot mode's second tap set costs a few spilled bytes at the largest
// radii), and the buckets above MP_VH_RMAX (256 threads, 1 CTA per SM: the
// larger window needs the registers, the wider strip keeps the halo share
// down).
#define MP_VH_KERNELS(NAME, CIN, CM) MP_VH_KERNELS_X(NAME, CIN, CM, vh_dispatch, 3, MP_VH_NT)
// Radius groups (see vh_dispatch_lo): 4 resident CTAs per SM for radii up to
// 8, 3 above.
#define MP_VH_KERNELS_LO(NAME, CIN, CM) MP_VH_KERNELS_X(NAME, CIN, CM, vh_dispatch_lo, 4, MP_VH_NT)
#define MP_VH_KERNELS_MID(NAME, CIN, CM) MP_VH_KERNELS_X(NAME, CIN, CM, vh_dispatch_mid, 4, MP_VH_NT)
#define MP_VH_KERNELS_HI(NAME, CIN, CM) MP_VH_KERNELS_X(NAME, CIN, CM, vh_dispatch_hi, 3, MP_VH_NT)
#define MP_VH_KERNELS_BIG(NAME, CIN, CM) MP_VH_KERNELS_X(NAME, CIN, CM, vh_dispatch_big, 1, MP_VH_NT_BIG)
#ifndef MP_VH_DOT_MINB
#define MP_VH_DOT_MINB 3
#endif
#define MP_VH_KERNELS_DOT(NAME, CIN, CM) MP_VH_KERNELS_X(NAME, CIN, CM, vh_dispatch_dot, MP_VH_DOT_MINB, MP_VH_NT)
