// mp_ops.cu -- per-op entry points (mpimg_*) and the batch pipeline planner.
//
// A pipeline (or a single op) is lowered per image into SEGMENTS.  A segment
// is one kernel launch kind (POINT, GAUSS, ROTATE, TRANSPOSE) with a
// pointwise prologue, a pointwise epilogue and an optional fliplr output map:
//   - pointwise ops (rgb2grey, brightness, adjust_gamma, colorize) join the
//     prologue of a segment that has no core yet, else its epilogue;
//   - fliplr sets the output map (pointwise ops commute with it);
//   - gaussian / rotate / transpose become the core of the current segment if
//     it has none and no flip yet, else they start a new segment.
// The reference applied each stage as a separate kernel with a fresh
// allocation and a stream sync in between (src/gpupipeline.c:373-397,
// src/millipyde_image.cpp:859-1142); here a 4-stage pipeline such as
// grey -> gaussian -> rotate -> gamma is two launches for the whole batch.
#include <math.h>
#include <string.h>
#include <stdlib.h>
#include <algorithm>
#include <mutex>
#include <vector>

#include "mp_internal.cuh"

// Reference degree->radian constant (src/millipyde_image.cpp:702).
#define MP_DEG2RAD 0.01745329252

// Intermediate bytes a chunk of a fused batch may hold (one launch per
// segment per chunk; mpk_tune_set_chunk_bytes changes it).  Measured on
// GB300: the uniform batch (256 x 1024^2 RGB) took 2.33 ms per step with
// 48 MB chunks and 1.49 ms with 512 MB; the ragged batch (1000 RGB images,
// 4 GB of intermediates) 6.59 ms with 512 MB and 6.06 ms with 2 GB (8 GB:
// the same) -- fewer, longer launches win over L2 residency.
static size_t mp_chunk_bytes = (size_t)2048 << 20;

struct ROp {
    int op;
    double p[3];
};

struct Seg {
    int kind;
    PwList pro, epi;
    int flip;
    int core_op;
    double core_p[3];
    int cin, cmid, cout;
    int hin, win, hout, wout;
    double rot_angle;   // FUSE: the rotate's angle (core_p holds the gaussian's sigma)
    PwList epi2;        // FUSE: the gaussian's epilogue
    int op0;            // index of the op that opened the segment (its input is a_op0)
};

// Fusion of a one-channel gaussian with the rotate after it (MPK_FUSE):
// 1 = on, 0 = off (default; mpk_tune_set_fuse, chosen by the autotuner from
// timings of both).
static int mp_fuse_mode = 0;

// Tuned geometry of the persistent kernels per launch kind (5 footprint
// rotate, 8 streaming gaussian, 9 fused gaussian + rotate), set by the
// autotuner through mpk_tune_set_kernel; 0 keeps the built-in choice.
enum { MP_TK_ITEMS = 0, MP_TK_CTAS = 1, MP_TK_STRIP = 2, MP_TK_NPARAM = 3 };
static int mp_ktune[16][MP_TK_NPARAM];
static std::mutex mp_ktune_mutex;

static int mp_tuned(int kind, int param)
{
    std::lock_guard<std::mutex> lk(mp_ktune_mutex);
    return mp_ktune[kind & 15][param];
}

// Resident CTAs per SM a persistent launch of `kind` uses: the occupancy
// limit, or the tuned cap when it is lower.
static int mp_cap_ctas(int kind, int cps)
{
    const int m = mp_tuned(kind, MP_TK_CTAS);
    return (m > 0 && m < cps) ? m : cps;
}

static bool mp_is_pointwise(int op)
{
    return op == MP_OP_RGB2GREY || op == MP_OP_BRIGHTNESS || op == MP_OP_ADJUST_GAMMA ||
           op == MP_OP_COLORIZE;
}

static int mp_round16(long long v) { return (int)((v + 15) / 16 * 16); }

// ---------------------------------------------------------------------------
// Parameter validation and resolution
// ---------------------------------------------------------------------------
static MPStatus mp_check_op(int op, const double *p)
{
    switch (op) {
    case MP_OP_RGB2GREY:
    case MP_OP_TRANSPOSE:
    case MP_OP_FLIPLR: return MILLIPYDE_SUCCESS;
    case MP_OP_GAUSSIAN:
        if (!(p[0] > 0.0) || !isfinite(p[0])) return MP_ERROR_INVALID_ARGS;
        if (ceil(3.0 * p[0]) > MP_MAX_RADIUS) return MP_ERROR_TOO_LARGE;
        return MILLIPYDE_SUCCESS;
    case MP_OP_ROTATE:
    case MP_OP_BRIGHTNESS: return isfinite(p[0]) ? MILLIPYDE_SUCCESS : MP_ERROR_INVALID_ARGS;
    case MP_OP_ADJUST_GAMMA:
        return (isfinite(p[0]) && isfinite(p[1])) ? MILLIPYDE_SUCCESS : MP_ERROR_INVALID_ARGS;
    case MP_OP_COLORIZE:
        return (p[0] >= 0 && p[1] >= 0 && p[2] >= 0 && isfinite(p[0]) && isfinite(p[1]) &&
                isfinite(p[2]))
                   ? MILLIPYDE_SUCCESS
                   : MP_ERROR_INVALID_ARGS;
    default: return MP_ERROR_BAD_DESCRIPTOR;
    }
}

static MPStatus mp_resolve_image(const MPStage *stages, int nstages, uint64_t seed, uint64_t index,
                                 std::vector<ROp> &ops, double *params_out)
{
    ops.clear();
    for (int s = 0; s < nstages; ++s) {
        const MPStage &st = stages[s];
        ROp r;
        r.op = st.op;
        for (int k = 0; k < 3; ++k) {
            if (st.random) {
                const double u = mp_counter_uniform(seed, index, (uint32_t)s, (uint32_t)k);
                r.p[k] = st.lo[k] + u * (st.hi[k] - st.lo[k]);
            } else {
                r.p[k] = st.lo[k];
            }
        }
        bool run = true;
        if (st.probability > 0.0 && st.probability < 1.0)
            run = mp_counter_uniform(seed, index, (uint32_t)s, 3u) <= st.probability;
        if (params_out) {
            for (int k = 0; k < 3; ++k) params_out[s * 4 + k] = r.p[k];
            params_out[s * 4 + 3] = run ? 1.0 : 0.0;
        }
        if (!run) continue;
        MPStatus c = mp_check_op(r.op, r.p);
        if (c != MILLIPYDE_SUCCESS) return c;
        ops.push_back(r);
    }
    return MILLIPYDE_SUCCESS;
}

// ---------------------------------------------------------------------------
// Segmentation
// ---------------------------------------------------------------------------
static void mp_pw_push(PwList &L, const ROp &r)
{
    PwOp o;
    o.op = r.op;
    o.p0 = (float)r.p[0];
    o.p1 = (float)(r.op == MP_OP_ADJUST_GAMMA ? r.p[1] : r.p[1]);
    o.p2 = (float)r.p[2];
    L.op[L.n++] = o;
}

static MPStatus mp_segment(const std::vector<ROp> &ops, int cin, int h, int w,
                           std::vector<Seg> &segs)
{
    segs.clear();
    Seg cur;
    memset(&cur, 0, sizeof(cur));
    cur.kind = MPK_POINT;
    cur.core_op = MP_OP_NONE;
    cur.cin = cur.cmid = cur.cout = cin;
    cur.hin = cur.hout = h;
    cur.win = cur.wout = w;
    int c = cin;
    int core_idx = -1;   // index of the current segment's core op
    for (size_t oi = 0; oi < ops.size(); ++oi) {
        const ROp &r = ops[oi];
        if (mp_is_pointwise(r.op)) {
            // identity cases: grey of a 1-channel image, colorize of a grey image
            if (r.op == MP_OP_RGB2GREY && c < 3) continue;
            if (r.op == MP_OP_COLORIZE && c < 3) continue;
            // rgb2grey after a colour gaussian, with no spatial op after it:
            // the grey starts a pointwise segment of its own.  The channel-
            // preserving streaming blur cannot reduce channels on its store,
            // and the tile kernel that can was slower than the streaming blur
            // plus a pointwise pass (64 x 512x512 RGB, sigma 1..3: 402 us
            // against about 200 + 60 us).  Without a flip in the gaussian's
            // segment its whole epilogue moves along: the pointwise pass costs
            // the same, and the segment boundary is then the blur's own
            // output, the intermediate a differentiable chain's backward
            // needs (saved by the forward instead of recomputed).
            if (r.op == MP_OP_RGB2GREY && cur.core_op == MP_OP_GAUSSIAN) {
                bool spatial_after = false;
                for (size_t q = oi + 1; q < ops.size(); ++q)
                    spatial_after = spatial_after || !(mp_is_pointwise(ops[q].op) || ops[q].op == MP_OP_FLIPLR);
                if (!spatial_after) {
                    Seg nx;
                    memset(&nx, 0, sizeof(nx));
                    nx.kind = MPK_POINT;
                    nx.core_op = MP_OP_NONE;
                    nx.cin = nx.cmid = nx.cout = c;
                    nx.hin = nx.hout = cur.hout;
                    nx.win = nx.wout = cur.wout;
                    nx.op0 = (int)oi;
                    if (!cur.flip && cur.epi.n > 0 && cur.epi.n < MP_MAX_PW) {
                        nx.pro = cur.epi;              // channel-preserving ops: c is unchanged
                        nx.op0 = core_idx + 1;
                        memset(&cur.epi, 0, sizeof(cur.epi));
                    }
                    segs.push_back(cur);
                    cur = nx;
                }
            }
            const bool to_pro = (cur.core_op == MP_OP_NONE && !cur.flip);
            PwList &L = to_pro ? cur.pro : cur.epi;
            if (L.n >= MP_MAX_PW) {
                // list full: close this segment and continue in a fresh one
                segs.push_back(cur);
                Seg nx;
                memset(&nx, 0, sizeof(nx));
                nx.kind = MPK_POINT;
                nx.cin = nx.cmid = nx.cout = c;
                nx.hin = nx.hout = cur.hout;
                nx.win = nx.wout = cur.wout;
                nx.op0 = (int)oi;
                cur = nx;
                mp_pw_push(cur.pro, r);
            } else {
                mp_pw_push(L, r);
            }
            if (r.op == MP_OP_RGB2GREY) c = 1;
            if (cur.core_op == MP_OP_NONE && !cur.flip && to_pro) cur.cmid = c;
            cur.cout = c;
            continue;
        }
        if (r.op == MP_OP_FLIPLR) {
            cur.flip ^= 1;
            continue;
        }
        // core op
        if (!(cur.core_op == MP_OP_NONE && !cur.flip)) {
            segs.push_back(cur);
            Seg nx;
            memset(&nx, 0, sizeof(nx));
            nx.cin = nx.cmid = nx.cout = c;
            nx.hin = nx.hout = cur.hout;
            nx.win = nx.wout = cur.wout;
            nx.op0 = (int)oi;
            cur = nx;
        }
        cur.core_op = r.op;
        core_idx = (int)oi;
        cur.core_p[0] = r.p[0];
        cur.core_p[1] = r.p[1];
        cur.core_p[2] = r.p[2];
        cur.cmid = c;
        cur.cout = c;
        if (r.op == MP_OP_GAUSSIAN) cur.kind = MPK_GAUSS;
        else if (r.op == MP_OP_ROTATE) cur.kind = MPK_ROTATE;
        else {
            cur.kind = MPK_TRANSPOSE;
            std::swap(cur.hout, cur.wout);
        }
    }
    segs.push_back(cur);
    return MILLIPYDE_SUCCESS;
}

// ---------------------------------------------------------------------------
// Job construction
// ---------------------------------------------------------------------------
static int mp_max_smem_optin()
{
    static int v = 0;
    if (!v) {
        int d = 0;
        cudaGetDevice(&d);
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, d) != cudaSuccess ||
            v <= 0) {
            cudaGetLastError();
            v = 227 * 1024;
        }
    }
    return v;
}

// Tile (tw, th) for a GAUSS launch: the largest candidate whose shared memory
// lets two CTAs share an SM, else the largest that fits at all.
// Autotuned gaussian tiles, set by mpk_tune_set_gauss_tile (the Python
// autotuner times candidate tiles on the device and records the fastest).
struct MPTuneEntry {
    int cin, cmid, has_pro, rlo, rhi, tw, th;
};
static std::vector<MPTuneEntry> mp_tune_table;
static std::mutex mp_tune_mutex;

static bool mp_gauss_tile_fits(int tw, int th, int r, int cin, int cmid, int has_pro)
{
    return tw >= 8 && th >= 8 && tw % 8 == 0 && th % 8 == 0 && th + 2 * r <= 256 &&
           mp_gauss_smem_bytes(tw, th, r, cin, cmid, has_pro) <= (size_t)mp_max_smem_optin();
}

static void mp_gauss_tiles(int r, int cin, int cmid, int has_pro, int *tw, int *th)
{
    {
        std::lock_guard<std::mutex> lk(mp_tune_mutex);
        for (const MPTuneEntry &e : mp_tune_table)
            if (e.cin == cin && e.cmid == cmid && e.has_pro == (has_pro ? 1 : 0) && r >= e.rlo &&
                r <= e.rhi && mp_gauss_tile_fits(e.tw, e.th, r, cin, cmid, has_pro)) {
                *tw = e.tw;
                *th = e.th;
                return;
            }
    }
    static const int grey[][2] = {{64, 64}, {128, 32}, {64, 32}, {64, 16}, {32, 16}, {16, 8}, {8, 8}};
    static const int colr[][2] = {{64, 32}, {32, 32}, {32, 16}, {16, 16}, {16, 8}, {8, 8}};
    const int(*cand)[2] = cmid == 1 ? grey : colr;
    const int nc = cmid == 1 ? 7 : 6;
    const size_t lim = (size_t)mp_max_smem_optin();
    for (int pass = 0; pass < 3; ++pass) {
        // prefer tiles that let 3 CTAs (the register limit) share an SM
        const size_t budget = pass == 0 ? lim / 3 - 1024 : pass == 1 ? lim / 2 - 1024 : lim;
        for (int i = 0; i < nc; ++i) {
            if (cand[i][1] + 2 * r > 256) continue;   // TMA box height limit
            if (mp_gauss_smem_bytes(cand[i][0], cand[i][1], r, cin, cmid, has_pro) <= budget) {
                *tw = cand[i][0];
                *th = cand[i][1];
                return;
            }
        }
    }
    *tw = 8;
    *th = 8;
}

static MPStatus mp_fill_job(MPJob &J, const Seg &sg, const MPImage &in, const MPImage &out, int tw,
                            int th)
{
    memset(&J, 0, sizeof(J));
    J.src = (const float *)in.data;
    J.dst = (float *)out.data;
    J.h = in.height;
    J.w = in.width;
    J.ho = out.height;
    J.wo = out.width;
    J.src_pitch = in.pitch / 4;
    J.dst_pitch = out.pitch / 4;
    J.cin = sg.cin;
    J.cmid = sg.cmid;
    J.cout = sg.cout;
    J.flip = sg.flip;
    J.pro = sg.pro;
    J.epi = sg.epi;
    switch (sg.kind) {
    case MPK_POINT:
        J.tiles_x = (in.width + 255) / 256;
        J.ntiles = J.tiles_x * ((in.height + 3) / 4);
        break;
    case MPK_ROTATE: {
        const double th_r = sg.core_p[0] * MP_DEG2RAD;
        const double scale = (double)(1LL << (MP_FIX_FRAC - 1));
        J.cosq = llround(cos(th_r) * scale);
        J.sinq = llround(sin(th_r) * scale);
        J.tiles_x = (out.width + 31) / 32;
        J.ntiles = J.tiles_x * ((out.height + 31) / 32);
        break;
    }
    case MPK_TRANSPOSE:
        J.tiles_x = (in.width + 31) / 32;
        J.ntiles = J.tiles_x * ((in.height + 31) / 32);
        break;
    case MPK_GAUSS: {
        const double sigma = sg.core_p[0];
        const int r = (int)ceil(3.0 * sigma);
        if (r < 1 || r > MP_MAX_RADIUS) return MP_ERROR_TOO_LARGE;
        J.radius = r;
        double e[MP_MAX_TAPS], sum = 0.0;
        for (int k = -r; k <= r; ++k) {
            e[k + r] = exp(-(double)(k * k) / (2.0 * sigma * sigma));
            sum += e[k + r];
        }
        for (int k = 0; k < 2 * r + 1; ++k) J.wts[k] = (float)(e[k] / sum);
        J.tw = tw;
        J.th = th;
        J.tiles_x = (in.width + tw - 1) / tw;
        J.ntiles = J.tiles_x * ((in.height + th - 1) / th);
        J.use_tma = 0;
        if ((in.pitch % 16) == 0 && (((uintptr_t)in.data) % 16) == 0 && in.width > 0 &&
            in.height > 0) {
            mp_encode_tiled_fn enc = mp_get_encode_tiled();
            if (enc) {
                cuuint64_t gdim[2] = {(cuuint64_t)in.width * (cuuint64_t)sg.cin,
                                      (cuuint64_t)in.height};
                cuuint64_t gstr[1] = {(cuuint64_t)in.pitch};
                cuuint32_t box[2] = {64u, (cuuint32_t)(th + 2 * r)};
                cuuint32_t es[2] = {1u, 1u};
                CUresult cr = enc(&J.tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)in.data, gdim,
                                  gstr, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
                if (cr == CUDA_SUCCESS) J.use_tma = 1;
            }
        }
        break;
    }
    default: return MP_ERROR_BAD_DESCRIPTOR;
    }
    return MILLIPYDE_SUCCESS;
}

// ---------------------------------------------------------------------------
// Streaming gaussian (mp_stream.cu) selection.
// ---------------------------------------------------------------------------
struct MPStreamTune {
    int cmid, ns;
};
static std::vector<MPStreamTune> mp_stream_tune;   // guarded by mp_tune_mutex

static int mp_num_sms()
{
    static int n = 0;
    if (!n) {
        int d = 0;
        cudaGetDevice(&d);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            n = 1;
        }
    }
    return n;
}

// A GAUSS segment runs on the streaming kernel when its source rows are
// TMA-legal (16-byte aligned base and pitch) and its epilogue keeps the
// channel count (no rgb2grey after the blur).
static bool mp_stream_ok(const Seg &sg, const MPImage &in)
{
    if (sg.kind != MPK_GAUSS || mp_variant(sg.cin, sg.cmid) < 0 || sg.cout != sg.cmid) return false;
    for (int i = 0; i < sg.epi.n; ++i)
        if (sg.epi.op[i].op == MP_OP_RGB2GREY) return false;
    if ((in.pitch % 16) || ((uintptr_t)in.data % 16) || in.width <= 0 || in.height <= 0) return false;
    return mp_get_encode_tiled() != nullptr;
}

// TMA stage count of the streaming gaussian for a channel count.
static int mp_stream_stages(int cmid)
{
    int ns = cmid == 1 ? 2 : 3;
    std::lock_guard<std::mutex> lk(mp_tune_mutex);
    for (const MPStreamTune &t : mp_stream_tune)
        if (t.cmid == cmid) ns = t.ns;
    return ns;
}

// Rows per strip item: about three items per resident CTA over the launch,
// at least 128 rows so the 2r halo rows stay a small share.
static int mp_stream_rows(long long strip_rows, int grid)
{
    const long long target = 3LL * (grid > 0 ? grid : 1);
    long long rs = (strip_rows + target - 1) / target;
    if (rs < 128) rs = 128;
    rs = (rs + 15) / 16 * 16;   // a multiple of every block height
    if (rs > (1 << 20)) rs = 1 << 20;
    return (int)rs;
}

static MPStatus mp_fill_job_stream(MPJob &J, const Seg &sg, const MPImage &in, const MPImage &out,
                                   int sw, int rs)
{
    memset(&J, 0, sizeof(J));
    J.src = (const float *)in.data;
    J.dst = (float *)out.data;
    J.h = in.height;
    J.w = in.width;
    J.ho = out.height;
    J.wo = out.width;
    J.src_pitch = in.pitch / 4;
    J.dst_pitch = out.pitch / 4;
    J.cin = sg.cin;
    J.cmid = sg.cmid;
    J.cout = sg.cout;
    J.flip = sg.flip;
    J.pro = sg.pro;
    J.epi = sg.epi;
    const double sigma = sg.core_p[0];
    const int r = (int)ceil(3.0 * sigma);
    if (r < 1 || r > MP_MAX_RADIUS) return MP_ERROR_TOO_LARGE;
    J.radius = r;
    double e[MP_MAX_TAPS], sum = 0.0;
    for (int k = -r; k <= r; ++k) {
        e[k + r] = exp(-(double)(k * k) / (2.0 * sigma * sigma));
        sum += e[k + r];
    }
    for (int k = 0; k < 2 * r + 1; ++k) J.wts[k] = (float)(e[k] / sum);
    J.tw = sw;
    J.th = rs;
    J.tiles_x = (in.width + sw - 1) / sw;
    J.ntiles = J.tiles_x * ((in.height + rs - 1) / rs);
    J.vec_out = (out.pitch % 16) == 0 && ((uintptr_t)out.data % 16) == 0;
    mp_encode_tiled_fn enc = mp_get_encode_tiled();
    if (!enc) return MP_ERROR_UNSUPPORTED_TYPE;
    cuuint64_t gdim[2] = {(cuuint64_t)in.width * (cuuint64_t)sg.cin, (cuuint64_t)in.height};
    cuuint64_t gstr[1] = {(cuuint64_t)in.pitch};
    cuuint32_t box[2] = {(cuuint32_t)mp_gs_boxw(sg.cin), (cuuint32_t)mp_gs_rb(sg.cmid)};
    cuuint32_t es[2] = {1u, 1u};
    CUresult cr = enc(&J.tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)in.data, gdim, gstr, box, es,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return MP_ERROR_UNSUPPORTED_TYPE;
    J.use_tma = 1;
    return MILLIPYDE_SUCCESS;
}

// Streaming launch geometry for a launch whose largest radius is rmax;
// false if the kernel cannot take it (the tile kernel runs instead).
static bool mp_stream_setup(int cin, int cmid, int rmax, GsGeom *g, int *grid)
{
    *g = mp_gs_geom(mp_stream_stages(cmid), mp_gs_bucket(rmax), cin, cmid);
    if ((size_t)g->total + 128 > (size_t)mp_max_smem_optin()) return false;
    int cps = 0;
    if (mp_gs_prepare(mp_variant(cin, cmid), (size_t)g->total + 128, &cps) != MILLIPYDE_SUCCESS) {
        cudaGetLastError();
        return false;
    }
    *grid = cps * mp_num_sms();
    return true;
}

// ---------------------------------------------------------------------------
// Footprint-staged rotate (mp_rot.cu) selection.
// ---------------------------------------------------------------------------
// A ROTATE segment runs on the footprint-staged kernel when it has no
// prologue and its source rows are TMA-legal.
static bool mp_rot_ok(const Seg &sg, const MPImage &in)
{
    if (sg.kind != MPK_ROTATE || sg.pro.n != 0 || sg.cin != sg.cmid) return false;
    if (sg.cin != 1 && sg.cin != 3 && sg.cin != 4) return false;
    if ((in.pitch % 16) || ((uintptr_t)in.data % 16) || in.width <= 0 || in.height <= 0) return false;
    return mp_get_encode_tiled() != nullptr;
}

static MPStatus mp_fill_job_rot(MPJob &J, const Seg &sg, const MPImage &in, const MPImage &out, bool adj = false,
                               int min_bxw = 0);

static MPStatus mp_fill_job_rot(MPJob &J, const Seg &sg, const MPImage &in, const MPImage &out, bool adj,
                               int min_bxw)
{
    MPStatus st = mp_fill_job(J, sg, in, out, 0, 0);   // source/destination, cos/sin, epilogue
    if (st != MILLIPYDE_SUCCESS) return st;
    const int C = sg.cin, TW = mp_ro_tw(C), TH = mp_ro_th(C);
    J.tiles_x = (out.width + TW - 1) / TW;
    J.ntiles = J.tiles_x * ((out.height + TH - 1) / TH);
    // footprint of a tile: the rotated tile's bounding box plus the bilinear
    // neighbour, in pixels; in floats plus up to 3 floats of alignment slack
    const double c = fabs((double)J.cosq) / (double)(1LL << (MP_FIX_FRAC - 1));
    const double sn = fabs((double)J.sinq) / (double)(1LL << (MP_FIX_FRAC - 1));
    // (+3: floor spread, bilinear neighbour, rounding; +1: the margin pixel
    // before the footprint).  The adjoint's box of g around a source tile
    // needs +7: two margin pixels before, the floor spread, three candidates
    // after the first, one pixel of float rounding.
    const int bw = (int)ceil((TW - 1) * c + (TH - 1) * sn + 1e-6) + (adj ? 7 : 4);
    const int bh = (int)ceil((TW - 1) * sn + (TH - 1) * c + 1e-6) + (adj ? 7 : 4);
    J.bxw = std::max((bw * C + 3 + 3) & ~3, min_bxw);
    J.byh = bh;
    if (J.bxw > 256 || J.byh > 256) return MP_ERROR_TOO_LARGE;
    mp_encode_tiled_fn enc = mp_get_encode_tiled();
    if (!enc) return MP_ERROR_UNSUPPORTED_TYPE;
    cuuint64_t gdim[2] = {(cuuint64_t)in.width * (cuuint64_t)C, (cuuint64_t)in.height};
    cuuint64_t gstr[1] = {(cuuint64_t)in.pitch};
    cuuint32_t box[2] = {(cuuint32_t)J.bxw, (cuuint32_t)J.byh};
    cuuint32_t es[2] = {1u, 1u};
    CUresult cr = enc(&J.tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)in.data, gdim, gstr, box, es,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return MP_ERROR_UNSUPPORTED_TYPE;
    J.use_tma = 1;
    return MILLIPYDE_SUCCESS;
}

static int mp_rot_buf_floats(const MPJob &J) { return (J.bxw * J.byh + 31) & ~31; }

// Row pitch (floats) of a footprint box padded against shared-memory bank
// conflicts.  The 32 lanes of a warp sample 32 consecutive output pixels
// of a row, which lie along a rotated line in the box; with a pitch that is
// a multiple of 32 floats a row step does not change the bank, and with
// one of 16 a step of two rows does not.  Modelled over angles in
// [-45, 45] degrees for 3 channels: about 1.6 shared-memory wavefronts per
// load at a multiple of 32, 2.0 at 16 mod 32, 2.4-2.6 at the other
// multiples of 4.  The padded box must fit the launch's buffer (`cap`
// floats) so that no job costs occupancy; 0 if no padding fits.
static int mp_rot_padded_bxw(const MPJob &J, int cap)
{
    const int p0 = (J.bxw + 31) & ~31;
    const int p16 = J.bxw <= 16 ? 16 : ((J.bxw - 16 + 31) & ~31) + 16;
    for (int p : {p0, p16})
        if (p <= 256 && ((p * J.byh + 31) & ~31) <= cap) return p;
    return 0;
}

// Persistent grid for a footprint-staged launch; false if it cannot run.
static bool mp_rot_setup(int c, int buf_floats, int *grid)
{
    const size_t smem = mp_ro_smem(buf_floats);
    if (smem > (size_t)mp_max_smem_optin()) return false;
    int cps = 0;
    if (mp_ro_prepare(c, smem, &cps) != MILLIPYDE_SUCCESS) {
        cudaGetLastError();
        return false;
    }
    *grid = mp_cap_ctas(MPK_RSTREAM, cps) * mp_num_sms();
    return true;
}

static void mp_seg_tiles(const Seg &sg, int *tw, int *th)
{
    *tw = *th = 0;
    if (sg.kind == MPK_GAUSS) {
        const int r = (int)ceil(3.0 * sg.core_p[0]);
        mp_gauss_tiles(r, sg.cin, sg.cmid, sg.pro.n > 0, tw, th);
    }
}

static size_t mp_seg_smem(const Seg &sg, int tw, int th)
{
    if (sg.kind != MPK_GAUSS) return 0;
    const int r = (int)ceil(3.0 * sg.core_p[0]);
    return mp_gauss_smem_bytes(tw, th, r, sg.cin, sg.cmid, sg.pro.n > 0);
}

// Runs one segment on one image with the job passed by value.
static MPStatus mp_vh_run_single(const Seg &sg, const MPImage &in, const MPImage &out, cudaStream_t s,
                                 bool *used);

static MPStatus mp_run_segment_single(const Seg &sg, const MPImage &in, const MPImage &out,
                                      cudaStream_t s)
{
    {
        bool used = false;
        MPStatus st = mp_vh_run_single(sg, in, out, s, &used);
        if (used || st != MILLIPYDE_SUCCESS) return st;
    }
    if (mp_rot_ok(sg, in)) {
        MPJob J;
        int grid = 0;
        if (mp_fill_job_rot(J, sg, in, out) == MILLIPYDE_SUCCESS && mp_rot_setup(sg.cin, mp_rot_buf_floats(J), &grid)) {
            int dev = 0;
            cudaGetDevice(&dev);
            int *err = mp_device_error_word(dev);
            if (!err) return MP_ERROR_NO_DEVICE;
            return mp_ro_launch_single(sg.cin, J, mp_rot_buf_floats(J), grid, err, s);
        }
    }
    if (mp_stream_ok(sg, in)) {
        GsGeom g;
        int grid;
        const int r = (int)ceil(3.0 * sg.core_p[0]);
        if (r >= 1 && r <= MP_MAX_RADIUS && mp_stream_setup(sg.cin, sg.cmid, r, &g, &grid)) {
            const long long strip_rows = (long long)((in.width + g.SW - 1) / g.SW) * in.height;
            MPJob J;
            MPStatus st = mp_fill_job_stream(J, sg, in, out, g.SW, mp_stream_rows(strip_rows, grid));
            if (st == MILLIPYDE_SUCCESS) {
                int dev = 0;
                cudaGetDevice(&dev);
                int *err = mp_device_error_word(dev);
                if (!err) return MP_ERROR_NO_DEVICE;
                return mp_gs_launch_single(mp_variant(sg.cin, sg.cmid), J, g, grid, err, s);
            }
        }
    }
    int tw, th;
    mp_seg_tiles(sg, &tw, &th);
    MPJob J;
    MPStatus st = mp_fill_job(J, sg, in, out, tw, th);
    if (st != MILLIPYDE_SUCCESS) return st;
    return mp_launch_single(sg.kind, J, mp_seg_smem(sg, tw, th), s);
}

// ---------------------------------------------------------------------------
// Plans: host-resolved job tables + launches (capturable in a CUDA graph).
// ---------------------------------------------------------------------------
struct MPLaunch {
    int kind;
    int variant;      // channel specialisation of GAUSS / ROTATE launches
    size_t job_off;   // first job of this launch in the job table
    size_t tile_off;  // first entry of this launch in the tile -> job map
    int njobs;
    int total_tiles;
    size_t smem;
    double bytes;   // algorithmic bytes: inputs read once + outputs written once
    int gauss[4];   // GAUSS: tile width, tile height, largest radius, all sources TMA-able
    GsGeom gs;      // GSTREAM: shared-memory geometry
    int grid;       // GSTREAM: persistent CTAs
    FzGeom fz;      // FUSE: shared-memory geometry
    int fz_cin;     // FUSE: source channels
};

struct MPPlanImpl {
    std::vector<MPLaunch> launches;
    void *tables = nullptr;    // one device block: job table, then tile -> job map
    MPJob *jobs_dev = nullptr;
    int *tiles_dev = nullptr;
    void *scratch = nullptr;
    int *counters = nullptr;   // one work counter per launch (dynamically scheduled kinds)
    int *err = nullptr;        // device error word the kernels report into
    int device = 0;
    cudaStream_t stream = nullptr;
};

// Kernel variant of a segment (channel specialisation for GAUSS / ROTATE).
static int mp_seg_variant(const Seg &sg)
{
    return (sg.kind == MPK_GAUSS || sg.kind == MPK_ROTATE || sg.kind == MPK_FUSE) ? mp_variant(sg.cin, sg.cmid) : 0;
}

static int mp_seg_key(const Seg &sg) { return sg.kind * 16 + mp_seg_variant(sg); }

// Host-side job table and tile -> job map of a plan under construction.
struct MPTables {
    std::vector<MPJob> jobs;
    std::vector<int> tiles;

    // Appends one launch made of the jobs in js (jobs with no tiles dropped).
    MPStatus add(std::vector<MPLaunch> &launches, int kind, int variant, size_t smem,
                 std::vector<MPJob> &js, double bytes)
    {
        MPLaunch L;
        memset(&L, 0, sizeof(L));
        L.kind = kind;
        L.variant = variant;
        L.job_off = jobs.size();
        L.tile_off = tiles.size();
        L.njobs = 0;
        L.total_tiles = 0;
        L.smem = smem;
        L.bytes = bytes;
        L.gauss[0] = L.gauss[1] = L.gauss[2] = 0;
        L.gauss[3] = 1;
        for (MPJob &J : js) {
            if (J.ntiles <= 0) continue;
            if ((long long)L.total_tiles + J.ntiles > 0x7fffffffLL) return MP_ERROR_TOO_LARGE;
            J.tile0 = L.total_tiles;
            L.total_tiles += J.ntiles;
            tiles.insert(tiles.end(), (size_t)J.ntiles, L.njobs);
            if (kind == MPK_GAUSS) {
                L.gauss[0] = J.tw;
                L.gauss[1] = J.th;
                L.gauss[2] = std::max(L.gauss[2], J.radius);
                L.gauss[3] &= J.use_tma;
            }
            jobs.push_back(J);
            L.njobs++;
        }
        if (L.njobs == 0) return MILLIPYDE_SUCCESS;
        if (kind < MPK_POINT_ADJ && kind != MPK_GSTREAM && kind != MPK_RSTREAM && kind != MPK_VH &&
            kind != MPK_RADJ && kind != MPK_RDTH && kind != MPK_FUSE) {
            MPStatus e = mp_prepare_kind(kind, variant, smem);
            if (e != MILLIPYDE_SUCCESS) return e;
        }
        launches.push_back(L);
        return MILLIPYDE_SUCCESS;
    }

    // One device block: jobs (128-byte aligned entries), then the tile map.
    MPStatus upload(MPPlanImpl *P, cudaStream_t s)
    {
        if (jobs.empty()) return MILLIPYDE_SUCCESS;
        const size_t jb = jobs.size() * sizeof(MPJob), tb = tiles.size() * sizeof(int);
        std::vector<unsigned char> host(jb + tb);
        memcpy(host.data(), jobs.data(), jb);
        memcpy(host.data() + jb, tiles.data(), tb);
        MPStatus st = mp_malloc_async(&P->tables, jb + tb, s);
        if (st != MILLIPYDE_SUCCESS) return st;
        P->jobs_dev = (MPJob *)P->tables;
        P->tiles_dev = (int *)((unsigned char *)P->tables + jb);
        return mp_upload_async(P->tables, host.data(), jb + tb, s);
    }
};

// ---------------------------------------------------------------------------
// Single-channel streaming gaussian (mp_vh.cuh) selection and jobs.
// ---------------------------------------------------------------------------
// A GAUSS segment runs on the mp_vh.cuh kernels when one of its families
// takes its channels (1 after the prologue, or C = 3 / 4 kept throughout),
// its radius is compiled there, its epilogue keeps the channel count and
// its source rows are TMA-legal.
static bool mp_vh_ok(const Seg &sg, const MPImage &in)
{
    const int r = (int)ceil(3.0 * sg.core_p[0]);
    if (sg.kind != MPK_GAUSS || mp_vh_code(sg.cin, sg.cmid, r) < 0 || sg.cout != sg.cmid) return false;
    for (int i = 0; i < sg.epi.n; ++i)
        if (sg.epi.op[i].op == MP_OP_RGB2GREY) return false;
    return (in.pitch % 16) == 0 && ((uintptr_t)in.data % 16) == 0 && in.width > 0 && in.height > 0 &&
           mp_get_encode_tiled() != nullptr;
}

static MPStatus mp_fill_job_vh(MPJob &J, const Seg &sg, const MPImage &in, const MPImage &out, int rs)
{
    MPStatus st = mp_fill_job(J, sg, in, out, 8, 8);   // radius, taps, pro/epilogue, flip
    if (st != MILLIPYDE_SUCCESS) return st;
    const int cm = (mp_vh_code(sg.cin, sg.cmid, J.radius) & 15) > 4 ? sg.cmid : 1;   // channels per column
    const int sw = mp_vh_fit_strip(mp_vh_bucket(J.radius), in.width, cm);           // in columns
    J.tw = sw;
    J.th = rs;
    J.tiles_x = (in.width * cm + sw - 1) / sw;
    J.ntiles = J.tiles_x * ((in.height + rs - 1) / rs);
    J.vec_out = (out.pitch % 16) == 0 && ((uintptr_t)out.data % 16) == 0;
    // source map: boxes of 64 columns x 8 rows (one per warp and staged group)
    mp_encode_tiled_fn enc = mp_get_encode_tiled();
    if (!enc) return MP_ERROR_UNSUPPORTED_TYPE;
    cuuint64_t gdim[2] = {(cuuint64_t)in.width * (cuuint64_t)sg.cin, (cuuint64_t)in.height};
    cuuint64_t gstr[1] = {(cuuint64_t)in.pitch};
    cuuint32_t box[2] = {(cuuint32_t)(64 * (cm == 1 ? sg.cin : 1)), 8u};
    cuuint32_t es[2] = {1u, 1u};
    CUresult cr = enc(&J.tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)in.data, gdim, gstr, box, es,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return MP_ERROR_UNSUPPORTED_TYPE;
    J.use_tma = 1;
    return MILLIPYDE_SUCCESS;
}

// Rows per strip item: about four items per resident CTA over the launch,
// at least 32 rows (the 2R head rows of an item are loads only).
static int mp_vh_rows(long long strip_rows, int grid)
{
    const int items = mp_tuned(MPK_VH, MP_TK_ITEMS);
    const long long target = (long long)(items > 0 ? items : 4) * (grid > 0 ? grid : 1);
    long long rs = (strip_rows + target - 1) / target;
    if (rs < 32) rs = 32;
    if (rs > 4096) rs = 4096;
    return (int)((rs + 7) / 8 * 8);
}

// One gaussian segment on one image with the single-channel kernel.
static MPStatus mp_vh_run_single(const Seg &sg, const MPImage &in, const MPImage &out, cudaStream_t s, bool *used)
{
    *used = false;
    if (!mp_vh_ok(sg, in)) return MILLIPYDE_SUCCESS;
    const int r = (int)ceil(3.0 * sg.core_p[0]);
    const int code = mp_vh_code(sg.cin, sg.cmid, r), cm = (code & 15) > 4 ? sg.cmid : 1;
    int cps = 0;
    if (mp_vh_prepare(code, &cps) != MILLIPYDE_SUCCESS) {
        cudaGetLastError();
        return MILLIPYDE_SUCCESS;
    }
    const int grid = mp_cap_ctas(MPK_VH, cps) * mp_num_sms();
    const int sw = mp_vh_fit_strip(mp_vh_bucket(r), in.width, cm);
    MPJob J;
    MPStatus st = mp_fill_job_vh(J, sg, in, out,
                                 mp_vh_rows((long long)((in.width * cm + sw - 1) / sw) * in.height, grid));
    if (st != MILLIPYDE_SUCCESS) return st;
    int dev = 0;
    cudaGetDevice(&dev);
    int *err = mp_device_error_word(dev);
    if (!err) return MP_ERROR_NO_DEVICE;
    *used = true;
    return mp_vh_launch_single(code, J, grid, err, s);
}

// Adds one launch of a rotate stage over images (sgs[i]: srcs[i] -> dsts[i])
// on the footprint-staged kernel when every image can take it; *added says
// whether it did (otherwise the caller builds the tile kernel's launch).
static MPStatus mp_add_rot(MPTables &T, std::vector<MPLaunch> &launches, const std::vector<Seg> &sgs,
                           const std::vector<MPImage> &srcs, const std::vector<MPImage> &dsts, bool *added)
{
    *added = false;
    if (sgs.empty()) return MILLIPYDE_SUCCESS;
    for (size_t i = 0; i < sgs.size(); ++i)
        if (!mp_rot_ok(sgs[i], srcs[i])) return MILLIPYDE_SUCCESS;
    std::vector<MPJob> js(sgs.size());
    double bytes = 0.0;
    int bufmax = 0;
    for (size_t i = 0; i < sgs.size(); ++i) {
        if (mp_fill_job_rot(js[i], sgs[i], srcs[i], dsts[i]) != MILLIPYDE_SUCCESS) return MILLIPYDE_SUCCESS;
        bufmax = std::max(bufmax, mp_rot_buf_floats(js[i]));
        bytes += 4.0 * ((double)srcs[i].height * srcs[i].width * srcs[i].channels +
                        (double)dsts[i].height * dsts[i].width * dsts[i].channels);
    }
    // boxes re-encoded with a bank-friendly pitch where it fits the buffer
    for (size_t i = 0; i < sgs.size(); ++i) {
        const int p = mp_rot_padded_bxw(js[i], bufmax);
        if (p > js[i].bxw && mp_fill_job_rot(js[i], sgs[i], srcs[i], dsts[i], false, p) != MILLIPYDE_SUCCESS)
            return MILLIPYDE_SUCCESS;
    }
    int grid = 0;
    const int c0 = sgs[0].cin;
    if (!mp_rot_setup(c0, bufmax, &grid)) return MILLIPYDE_SUCCESS;
    const size_t nl = launches.size();
    MPStatus st = T.add(launches, MPK_RSTREAM, c0, mp_ro_smem(bufmax), js, bytes);
    if (st != MILLIPYDE_SUCCESS) return st;
    if (launches.size() > nl) {
        launches.back().grid = grid;
        launches.back().gauss[0] = bufmax;
    }
    *added = true;
    return MILLIPYDE_SUCCESS;
}

// Adds one launch of a gaussian stage over images (sgs[i]: srcs[i] ->
// dsts[i]) with the fastest kernel that takes every image: the mp_vh.cuh
// streaming kernels, the strip-streaming kernel, else the tile kernel.  The
// images go into the job table in order of radius: work items are handed out
// in table order, so the CTAs of an SM run one compiled radius at a time
// instead of thrashing the instruction cache with all of them.
static MPStatus mp_add_gauss_ordered(MPTables &T, std::vector<MPLaunch> &launches, const std::vector<Seg> &sgs,
                                     const std::vector<MPImage> &srcs, const std::vector<MPImage> &dsts);

static MPStatus mp_add_gauss(MPTables &T, std::vector<MPLaunch> &launches, const std::vector<Seg> &sgs,
                             const std::vector<MPImage> &srcs, const std::vector<MPImage> &dsts)
{
    std::vector<size_t> ord(sgs.size());
    for (size_t i = 0; i < ord.size(); ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
        return (int)ceil(3.0 * sgs[a].core_p[0]) < (int)ceil(3.0 * sgs[b].core_p[0]);
    });
    std::vector<Seg> s2;
    std::vector<MPImage> i2, o2;
    for (size_t i : ord) {
        s2.push_back(sgs[i]);
        i2.push_back(srcs[i]);
        o2.push_back(dsts[i]);
    }
    return mp_add_gauss_ordered(T, launches, s2, i2, o2);
}

static MPStatus mp_add_gauss_ordered(MPTables &T, std::vector<MPLaunch> &launches, const std::vector<Seg> &sgs,
                                     const std::vector<MPImage> &srcs, const std::vector<MPImage> &dsts)
{
    if (sgs.empty()) return MILLIPYDE_SUCCESS;
    const Seg &s0 = sgs[0];
    const size_t n = sgs.size();
    double bytes = 0.0;
    int rmax = 1;
    bool vh = true, gs = true;
    long long gs_rows = 0;
    std::vector<int> code(n);
    for (size_t i = 0; i < n; ++i) {
        const int r = (int)ceil(3.0 * sgs[i].core_p[0]);
        rmax = std::max(rmax, r);
        code[i] = mp_vh_code(sgs[i].cin, sgs[i].cmid, r);
        vh = vh && mp_vh_ok(sgs[i], srcs[i]);
        gs = gs && mp_stream_ok(sgs[i], srcs[i]);
        bytes += 4.0 * ((double)srcs[i].height * srcs[i].width * srcs[i].channels +
                        (double)dsts[i].height * dsts[i].width * dsts[i].channels);
    }
    MPStatus st;
    // mp_vh.cuh kernels: one launch per kernel code (radius order keeps each
    // code's images together); every code is prepared before any is added
    std::vector<std::pair<size_t, size_t>> runs;
    std::vector<int> grids;
    for (size_t a = 0; vh && a < n;) {
        size_t b = a + 1;
        while (b < n && code[b] == code[a]) ++b;
        int cps = 0;
        if (mp_vh_prepare(code[a], &cps) != MILLIPYDE_SUCCESS) vh = false;
        runs.push_back({a, b});
        grids.push_back(mp_cap_ctas(MPK_VH, cps) * mp_num_sms());
        a = b;
    }
    if (vh) {
        for (size_t q = 0; q < runs.size(); ++q) {
            const size_t a = runs[q].first, b = runs[q].second;
            const int cm = (code[a] & 15) > 4 ? sgs[a].cmid : 1;
            long long vh_rows = 0;
            double rb = 0.0;
            for (size_t i = a; i < b; ++i) {
                const int sw = mp_vh_fit_strip(mp_vh_bucket((int)ceil(3.0 * sgs[i].core_p[0])), srcs[i].width, cm);
                vh_rows += (long long)((srcs[i].width * cm + sw - 1) / sw) * srcs[i].height;
                rb += 4.0 * ((double)srcs[i].height * srcs[i].width * srcs[i].channels +
                             (double)dsts[i].height * dsts[i].width * dsts[i].channels);
            }
            const int rs = mp_vh_rows(vh_rows, grids[q]);
            std::vector<MPJob> js(b - a);
            for (size_t i = a; i < b; ++i) {
                st = mp_fill_job_vh(js[i - a], sgs[i], srcs[i], dsts[i], rs);
                if (st != MILLIPYDE_SUCCESS) return st;
            }
            const size_t nl = launches.size();
            st = T.add(launches, MPK_VH, code[a], 0, js, rb);
            if (st != MILLIPYDE_SUCCESS) return st;
            if (launches.size() > nl) launches.back().grid = grids[q];
        }
        return MILLIPYDE_SUCCESS;
    }
    cudaGetLastError();
    GsGeom g;
    int grid = 0;
    if (gs && rmax <= MP_MAX_RADIUS && mp_stream_setup(s0.cin, s0.cmid, rmax, &g, &grid)) {
        for (size_t i = 0; i < sgs.size(); ++i)
            gs_rows += (long long)((srcs[i].width + g.SW - 1) / g.SW) * srcs[i].height;
        const int rs = mp_stream_rows(gs_rows, grid);
        std::vector<MPJob> js(sgs.size());
        for (size_t i = 0; i < sgs.size(); ++i) {
            st = mp_fill_job_stream(js[i], sgs[i], srcs[i], dsts[i], g.SW, rs);
            if (st != MILLIPYDE_SUCCESS) return st;
        }
        const size_t nl = launches.size();
        st = T.add(launches, MPK_GSTREAM, mp_variant(s0.cin, s0.cmid), (size_t)g.total + 128, js, bytes);
        if (st == MILLIPYDE_SUCCESS && launches.size() > nl) {
            launches.back().gs = g;
            launches.back().grid = grid;
        }
        return st;
    }
    // tile kernel
    int tw, th, cinm = 1, cmidm = 1, pro = 0;
    for (const Seg &sg : sgs) {
        cinm = std::max(cinm, sg.cin);
        cmidm = std::max(cmidm, sg.cmid);
        pro |= sg.pro.n > 0;
    }
    mp_gauss_tiles(rmax, cinm, cmidm, pro, &tw, &th);
    const size_t smem = mp_gauss_smem_bytes(tw, th, rmax, cinm, cmidm, pro);
    std::vector<MPJob> js(sgs.size());
    for (size_t i = 0; i < sgs.size(); ++i) {
        st = mp_fill_job(js[i], sgs[i], srcs[i], dsts[i], tw, th);
        if (st != MILLIPYDE_SUCCESS) return st;
    }
    return T.add(launches, MPK_GAUSS, mp_variant(s0.cin, s0.cmid), smem, js, bytes);
}

// ---------------------------------------------------------------------------
// Fused gaussian -> rotate (mp_fuse.cuh).
// ---------------------------------------------------------------------------
// Merges a one-channel gaussian segment and the rotate segment after it into
// one FUSE segment when the fused kernel takes them: the blur keeps one
// channel and has no mirror map, its radius is compiled there, the rotate
// has no prologue, and the gaussian's source rows are TMA-legal (`in` is the
// first segment's source; later sources are the plan's own intermediates,
// always 16-byte aligned).
static void mp_fuse_segments(std::vector<Seg> &segs, const MPImage &in)
{
    if (!mp_fuse_mode || !mp_get_encode_tiled()) return;
    for (size_t k = 0; k + 1 < segs.size(); ++k) {
        const Seg &g = segs[k], &r = segs[k + 1];
        if (g.kind != MPK_GAUSS || r.kind != MPK_ROTATE) continue;
        const int rad = (int)ceil(3.0 * g.core_p[0]);
        if (g.cmid != 1 || g.cout != 1 || g.flip || !mp_fz_supported(g.cin, rad)) continue;
        if (r.pro.n != 0 || r.cin != 1 || r.cmid != 1) continue;
        if (k == 0 && ((in.pitch % 16) || ((uintptr_t)in.data % 16) || in.width <= 0 || in.height <= 0)) continue;
        Seg f = g;
        f.kind = MPK_FUSE;
        f.epi2 = g.epi;
        f.epi = r.epi;
        f.flip = r.flip;
        f.rot_angle = r.core_p[0];
        f.cout = r.cout;
        f.hout = r.hout;
        f.wout = r.wout;
        segs[k] = f;
        segs.erase(segs.begin() + (long)k + 1);
    }
}

// Footprint box (pixels) of a 64 x 64 output tile rotated by `angle`
// degrees: the rotated tile's bounding box plus the bilinear neighbour and
// the rounding margins of the rotate kernel (mp_fill_job_rot).
static int mp_fz_box(double angle)
{
    const double th = angle * MP_DEG2RAD;
    return (int)ceil(63.0 * fabs(cos(th)) + 63.0 * fabs(sin(th)) + 1e-6) + 4;
}

static MPStatus mp_fill_job_fuse(MPJob &J, const Seg &sg, const MPImage &in, const MPImage &out)
{
    memset(&J, 0, sizeof(J));
    J.src = (const float *)in.data;
    J.dst = (float *)out.data;
    J.h = in.height;
    J.w = in.width;
    J.ho = out.height;
    J.wo = out.width;
    J.src_pitch = in.pitch / 4;
    J.dst_pitch = out.pitch / 4;
    J.cin = sg.cin;
    J.cmid = 1;
    J.cout = sg.cout;
    J.flip = sg.flip;
    J.pro = sg.pro;
    J.epi = sg.epi;
    J.epi2 = sg.epi2;
    const double sigma = sg.core_p[0];
    const int r = (int)ceil(3.0 * sigma);
    if (r < 1 || r > MP_FZ_RMAX) return MP_ERROR_TOO_LARGE;
    J.radius = r;
    double e[MP_MAX_TAPS], sum = 0.0;
    for (int k = -r; k <= r; ++k) {
        e[k + r] = exp(-(double)(k * k) / (2.0 * sigma * sigma));
        sum += e[k + r];
    }
    for (int k = 0; k < 2 * r + 1; ++k) J.wts[k] = (float)(e[k] / sum);
    const double th_r = sg.rot_angle * MP_DEG2RAD;
    const double scale = (double)(1LL << (MP_FIX_FRAC - 1));
    J.cosq = llround(cos(th_r) * scale);
    J.sinq = llround(sin(th_r) * scale);
    J.tw = J.th = 64;
    J.tiles_x = (out.width + 63) / 64;
    J.ntiles = J.tiles_x * ((out.height + 63) / 64);
    J.bxw = J.byh = mp_fz_box(sg.rot_angle);
    mp_encode_tiled_fn enc = mp_get_encode_tiled();
    if (!enc) return MP_ERROR_UNSUPPORTED_TYPE;
    cuuint64_t gdim[2] = {(cuuint64_t)in.width * (cuuint64_t)sg.cin, (cuuint64_t)in.height};
    cuuint64_t gstr[1] = {(cuuint64_t)in.pitch};
    cuuint32_t box[2] = {128u, (cuuint32_t)MP_FZ_CR};
    cuuint32_t es[2] = {1u, 1u};
    CUresult cr = enc(&J.tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)in.data, gdim, gstr, box, es,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return MP_ERROR_UNSUPPORTED_TYPE;
    J.use_tma = 1;
    return MILLIPYDE_SUCCESS;
}

// One FUSE launch over images (sgs[i]: srcs[i] -> dsts[i]), jobs in radius
// order (an SM's CTAs then run one compiled radius at a time).
static MPStatus mp_add_fuse(MPTables &T, std::vector<MPLaunch> &launches, const std::vector<Seg> &sgs,
                            const std::vector<MPImage> &srcs, const std::vector<MPImage> &dsts)
{
    if (sgs.empty()) return MILLIPYDE_SUCCESS;
    std::vector<size_t> ord(sgs.size());
    for (size_t i = 0; i < ord.size(); ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return sgs[a].core_p[0] < sgs[b].core_p[0]; });
    std::vector<MPJob> js(sgs.size());
    double bytes = 0.0;
    int box_max = 0, rmax = 1;
    for (size_t q = 0; q < ord.size(); ++q) {
        const size_t i = ord[q];
        MPStatus st = mp_fill_job_fuse(js[q], sgs[i], srcs[i], dsts[i]);
        if (st != MILLIPYDE_SUCCESS) return st;
        box_max = std::max(box_max, js[q].bxw);
        rmax = std::max(rmax, js[q].radius);
        bytes += 4.0 * ((double)srcs[i].height * srcs[i].width * srcs[i].channels +
                        (double)dsts[i].height * dsts[i].width * dsts[i].channels);
    }
    const int cin = sgs[0].cin;
    size_t smem = 0;
    const FzGeom g = mp_fz_geom(box_max, rmax, cin, &smem);
    int cps = 0;
    MPStatus st = mp_fz_prepare(cin, smem, &cps);
    if (st != MILLIPYDE_SUCCESS) return st;
    const size_t nl = launches.size();
    st = T.add(launches, MPK_FUSE, mp_variant(cin, 1), smem, js, bytes);
    if (st != MILLIPYDE_SUCCESS) return st;
    if (launches.size() > nl) {
        launches.back().grid = mp_cap_ctas(MPK_FUSE, cps) * mp_num_sms();
        launches.back().fz = g;
        launches.back().fz_cin = cin;
    }
    return MILLIPYDE_SUCCESS;
}

// Job table upload plus the per-launch work counters of a plan.
static MPStatus mp_plan_finish(MPPlanImpl *P, MPTables &T, cudaStream_t s)
{
    MPStatus st = T.upload(P, s);
    if (st != MILLIPYDE_SUCCESS || P->launches.empty()) return st;
    const size_t cb = P->launches.size() * sizeof(int);
    st = mp_malloc_async((void **)&P->counters, cb, s);
    if (st != MILLIPYDE_SUCCESS) return st;
    return mp_cuda_status(cudaMemsetAsync(P->counters, 0, cb, s));
}

// Caller-provided homes for a plan's intermediates (the saved forward
// intermediates of a differentiable chain): image i's output of segment s
// (s below its last) is written to at[i][s] when at[i][s].data is set, and
// takes no scratch.  Plans with homes skip fusion, so that every segment
// boundary stays materialised.
struct MPInterHomes {
    std::vector<std::vector<MPImage>> at;
    bool has(int i, size_t s) const { return i < (int)at.size() && s < at[i].size() && at[i][s].data; }
};

static MPStatus mp_plan_build(const MPStage *stages, int nstages, const MPImage *in,
                              const MPImage *out, int nimgs, uint64_t seed, uint64_t index0,
                              cudaStream_t s, MPPlanImpl *P,
                              const std::vector<std::vector<ROp>> *explicit_ops = nullptr,
                              const MPInterHomes *homes = nullptr)
{
    if (nimgs < 0 || nstages < 0 || (nimgs > 0 && (!in || !out)) ||
        (nstages > 0 && !stages && !explicit_ops))
        return MP_ERROR_BAD_DESCRIPTOR;
    // device set-up (error word, pool) happens here, never during a capture
    P->err = mp_device_error_word(P->device);
    if (!P->err) return MP_ERROR_NO_DEVICE;
    // 1. resolve + segment every image
    std::vector<std::vector<Seg>> segs(nimgs);
    std::vector<ROp> ops;
    for (int i = 0; i < nimgs; ++i) {
        if (in[i].height < 0 || in[i].width < 0 || in[i].pitch < 0 || (in[i].pitch % 4) ||
            (in[i].channels != 1 && in[i].channels != 3 && in[i].channels != 4))
            return MP_ERROR_BAD_DESCRIPTOR;
        if ((long long)in[i].width * in[i].channels * 4 > in[i].pitch && in[i].height > 0)
            return MP_ERROR_BAD_DESCRIPTOR;
        if (explicit_ops) {
            ops = (*explicit_ops)[i];
            for (const ROp &r : ops) {
                MPStatus c = mp_check_op(r.op, r.p);
                if (c != MILLIPYDE_SUCCESS) return c;
            }
        } else {
            MPStatus st = mp_resolve_image(stages, nstages, seed, index0 + (uint64_t)i, ops, nullptr);
            if (st != MILLIPYDE_SUCCESS) return st;
        }
        mp_segment(ops, in[i].channels, in[i].height, in[i].width, segs[i]);
        if (!homes) mp_fuse_segments(segs[i], in[i]);
        const Seg &last = segs[i].back();
        if (!out[i].data && (long long)last.hout * last.wout > 0) return MP_ERROR_NULL_DATA;
        if (out[i].height != last.hout || out[i].width != last.wout ||
            out[i].channels != last.cout || out[i].pitch < last.wout * last.cout * 4 ||
            (out[i].pitch % 4))
            return MP_ERROR_BAD_DESCRIPTOR;
    }
    // 2. group images by their sequence of segment kinds (keeps batch order
    //    within a group), then chunk each group so intermediates stay in L2.
    std::vector<int> order(nimgs);
    for (int i = 0; i < nimgs; ++i) order[i] = i;
    auto sig_less = [&](int a, int b) {
        const auto &A = segs[a], &B = segs[b];
        if (A.size() != B.size()) return A.size() < B.size();
        for (size_t k = 0; k < A.size(); ++k)
            if (mp_seg_key(A[k]) != mp_seg_key(B[k])) return mp_seg_key(A[k]) < mp_seg_key(B[k]);
        return a < b;
    };
    std::sort(order.begin(), order.end(), sig_less);

    struct Chunk { std::vector<int> imgs; };
    std::vector<Chunk> chunks;
    size_t scratch_need = 0;
    {
        size_t i = 0;
        while (i < order.size()) {
            Chunk ch;
            size_t bytes = 0;
            const auto &sig0 = segs[order[i]];
            while (i < order.size()) {
                const auto &sg = segs[order[i]];
                bool same = sg.size() == sig0.size();
                for (size_t k = 0; same && k < sg.size(); ++k) same = mp_seg_key(sg[k]) == mp_seg_key(sig0[k]);
                if (!same) break;
                size_t b = 0;
                for (size_t k = 0; k + 1 < sg.size(); ++k)
                    if (!homes || !homes->has(order[i], k))
                        b += (size_t)sg[k].hout * mp_round16((long long)sg[k].wout * sg[k].cout * 4);
                if (!ch.imgs.empty() && bytes + b > mp_chunk_bytes) break;
                bytes += b;
                ch.imgs.push_back(order[i]);
                ++i;
            }
            scratch_need = std::max(scratch_need, bytes);
            chunks.push_back(ch);
        }
    }
    // 3. scratch for intermediates (reused by every chunk, stream-ordered)
    MPStatus st = mp_malloc_async(&P->scratch, scratch_need, s);
    if (st != MILLIPYDE_SUCCESS) return st;
    // 4. jobs
    MPTables T;
    for (const Chunk &ch : chunks) {
        const size_t nseg = segs[ch.imgs[0]].size();
        // intermediate images of this chunk
        std::vector<std::vector<MPImage>> inter(ch.imgs.size(), std::vector<MPImage>(nseg));
        size_t off = 0;
        for (size_t q = 0; q < ch.imgs.size(); ++q) {
            const auto &sg = segs[ch.imgs[q]];
            for (size_t k = 0; k + 1 < nseg; ++k) {
                if (homes && homes->has(ch.imgs[q], k)) {
                    inter[q][k] = homes->at[ch.imgs[q]][k];
                    continue;
                }
                MPImage m;
                m.height = sg[k].hout;
                m.width = sg[k].wout;
                m.channels = sg[k].cout;
                m.pitch = mp_round16((long long)m.width * m.channels * 4);
                m.data = (char *)P->scratch + off;
                off += (size_t)m.height * m.pitch;
                inter[q][k] = m;
            }
        }
        for (size_t k = 0; k < nseg; ++k) {
            // uniform tile geometry for this launch
            int kind = segs[ch.imgs[0]][k].kind;
            int tw = 0, th = 0;
            size_t smem = 0;
            if (kind == MPK_FUSE) {
                std::vector<Seg> sgs;
                std::vector<MPImage> srcs, dsts;
                for (size_t q = 0; q < ch.imgs.size(); ++q) {
                    const int img = ch.imgs[q];
                    sgs.push_back(segs[img][k]);
                    srcs.push_back((k == 0) ? in[img] : inter[q][k - 1]);
                    dsts.push_back((k + 1 == nseg) ? out[img] : inter[q][k]);
                }
                st = mp_add_fuse(T, P->launches, sgs, srcs, dsts);
                if (st != MILLIPYDE_SUCCESS) return st;
                continue;
            }
            if (kind == MPK_ROTATE) {
                std::vector<Seg> sgs;
                std::vector<MPImage> srcs, dsts;
                for (size_t q = 0; q < ch.imgs.size(); ++q) {
                    const int img = ch.imgs[q];
                    sgs.push_back(segs[img][k]);
                    srcs.push_back((k == 0) ? in[img] : inter[q][k - 1]);
                    dsts.push_back((k + 1 == nseg) ? out[img] : inter[q][k]);
                }
                bool added = false;
                st = mp_add_rot(T, P->launches, sgs, srcs, dsts, &added);
                if (st != MILLIPYDE_SUCCESS) return st;
                if (added) continue;
            }
            if (kind == MPK_GAUSS) {
                std::vector<Seg> sgs;
                std::vector<MPImage> srcs, dsts;
                for (size_t q = 0; q < ch.imgs.size(); ++q) {
                    const int img = ch.imgs[q];
                    sgs.push_back(segs[img][k]);
                    srcs.push_back((k == 0) ? in[img] : inter[q][k - 1]);
                    dsts.push_back((k + 1 == nseg) ? out[img] : inter[q][k]);
                }
                st = mp_add_gauss(T, P->launches, sgs, srcs, dsts);
                if (st != MILLIPYDE_SUCCESS) return st;
                continue;
            }
            std::vector<MPJob> js;
            double bytes = 0.0;
            for (size_t q = 0; q < ch.imgs.size(); ++q) {
                const int img = ch.imgs[q];
                const Seg &sg = segs[img][k];
                const MPImage &src = (k == 0) ? in[img] : inter[q][k - 1];
                const MPImage &dst = (k + 1 == nseg) ? out[img] : inter[q][k];
                MPJob J;
                st = mp_fill_job(J, sg, src, dst, tw, th);
                if (st != MILLIPYDE_SUCCESS) return st;
                bytes += 4.0 * ((double)src.height * src.width * src.channels +
                                (double)dst.height * dst.width * dst.channels);
                js.push_back(J);
            }
            st = T.add(P->launches, kind, mp_seg_variant(segs[ch.imgs[0]][k]), smem, js, bytes);
            if (st != MILLIPYDE_SUCCESS) return st;
        }
    }
    return mp_plan_finish(P, T, s);
}

static MPStatus mp_plan_launch_one(const MPPlanImpl *P, size_t idx, cudaStream_t s)
{
    const MPLaunch &L = P->launches[idx];
    if (L.kind >= MPK_POINT_ADJ)
        return mp_launch_adjoint(L.kind, P->jobs_dev + L.job_off, P->tiles_dev + L.tile_off, L.total_tiles,
                                 P->err, s);
    if (L.kind == MPK_VH) {
        // items beyond the first one per CTA are handed out by a counter,
        // zeroed before every launch (a memset node under graph capture)
        MPStatus st = mp_cuda_status(cudaMemsetAsync(P->counters + idx, 0, sizeof(int), s));
        if (st != MILLIPYDE_SUCCESS) return st;
        return mp_vh_launch(L.variant, P->jobs_dev + L.job_off, P->tiles_dev + L.tile_off, L.total_tiles, L.grid,
                            P->err, P->counters + idx, s);
    }
    if (L.kind == MPK_FUSE)
        return mp_fz_launch(L.fz_cin, P->jobs_dev + L.job_off, P->tiles_dev + L.tile_off, L.total_tiles, L.fz, L.smem,
                            L.grid, P->err, s);
    if (L.kind == MPK_RSTREAM || L.kind == MPK_RADJ || L.kind == MPK_RDTH)
        return mp_ro_launch(L.variant, P->jobs_dev + L.job_off, P->tiles_dev + L.tile_off, L.total_tiles,
                            L.gauss[0], L.grid, P->err, s);
    if (L.kind == MPK_GSTREAM)
        return mp_gs_launch(L.variant, P->jobs_dev + L.job_off, P->tiles_dev + L.tile_off, L.total_tiles, L.gs,
                            L.grid, P->err, s);
    return mp_launch_kind(L.kind, L.variant, P->jobs_dev + L.job_off, P->tiles_dev + L.tile_off, L.total_tiles,
                          L.smem, P->err, s, L.gauss);
}

static MPStatus mp_plan_launch(const MPPlanImpl *P, cudaStream_t s)
{
    for (size_t i = 0; i < P->launches.size(); ++i) {
        MPStatus st = mp_plan_launch_one(P, i, s);
        if (st != MILLIPYDE_SUCCESS) return st;
    }
    return MILLIPYDE_SUCCESS;
}

static void mp_plan_free(MPPlanImpl *P, cudaStream_t s)
{
    mp_free_async(P->tables, s);
    mp_free_async(P->scratch, s);
    mp_free_async(P->counters, s);
    P->counters = nullptr;
    P->tables = nullptr;
    P->jobs_dev = nullptr;
    P->tiles_dev = nullptr;
    P->scratch = nullptr;
}

extern "C" {

MPStatus mpk_plan_create(const MPStage *stages, int nstages, const MPImage *in, const MPImage *out,
                         int nimgs, uint64_t seed, uint64_t index0, void *stream, MPPlan **plan)
{
    if (!plan) return MP_ERROR_INVALID_ARGS;
    *plan = nullptr;
    MPPlanImpl *P = new (std::nothrow) MPPlanImpl();
    if (!P) return MP_ERROR_OUT_OF_MEMORY;
    cudaGetDevice(&P->device);
    P->stream = (cudaStream_t)stream;
    MPStatus st = mp_plan_build(stages, nstages, in, out, nimgs, seed, index0, P->stream, P);
    if (st != MILLIPYDE_SUCCESS) {
        mp_plan_free(P, P->stream);
        delete P;
        return st;
    }
    *plan = (MPPlan *)P;
    return MILLIPYDE_SUCCESS;
}

MPStatus mpk_plan_launch(MPPlan *plan, void *stream)
{
    if (!plan) return MP_ERROR_INVALID_ARGS;
    return mp_plan_launch((MPPlanImpl *)plan, (cudaStream_t)stream);
}

int mpk_plan_num_launches(const MPPlan *plan)
{
    return plan ? (int)((const MPPlanImpl *)plan)->launches.size() : 0;
}

MPStatus mpk_plan_launch_range(MPPlan *plan, int first, int count, void *stream)
{
    if (!plan) return MP_ERROR_INVALID_ARGS;
    const MPPlanImpl *P = (const MPPlanImpl *)plan;
    if (first < 0 || count < 0 || first + count > (int)P->launches.size()) return MP_ERROR_INVALID_ARGS;
    for (int i = first; i < first + count; ++i) {
        MPStatus st = mp_plan_launch_one(P, (size_t)i, (cudaStream_t)stream);
        if (st != MILLIPYDE_SUCCESS) return st;
    }
    return MILLIPYDE_SUCCESS;
}

MPStatus mpk_plan_launch_info(const MPPlan *plan, int i, int *kind, int *njobs, int *tiles,
                              double *bytes)
{
    if (!plan) return MP_ERROR_INVALID_ARGS;
    const MPPlanImpl *P = (const MPPlanImpl *)plan;
    if (i < 0 || i >= (int)P->launches.size()) return MP_ERROR_INVALID_ARGS;
    const MPLaunch &L = P->launches[i];
    if (kind) *kind = L.kind;
    if (njobs) *njobs = L.njobs;
    if (tiles) *tiles = L.total_tiles;
    if (bytes) *bytes = L.bytes;
    return MILLIPYDE_SUCCESS;
}

MPStatus mpk_plan_destroy(MPPlan *plan)
{
    if (!plan) return MILLIPYDE_SUCCESS;
    MPPlanImpl *P = (MPPlanImpl *)plan;
    mp_plan_free(P, P->stream);
    delete P;
    return MILLIPYDE_SUCCESS;
}

MPStatus mpk_pipeline_resolve(const MPStage *stages, int nstages, int nimgs, uint64_t seed,
                              uint64_t index0, double *params)
{
    if (nimgs < 0 || nstages < 0 || !params) return MP_ERROR_INVALID_ARGS;
    std::vector<ROp> ops;
    for (int i = 0; i < nimgs; ++i) {
        MPStatus st =
            mp_resolve_image(stages, nstages, seed, index0 + (uint64_t)i, ops, params + (size_t)i * nstages * 4);
        if (st != MILLIPYDE_SUCCESS) return st;
    }
    return MILLIPYDE_SUCCESS;
}

MPStatus mpk_pipeline_shapes(const MPStage *stages, int nstages, const MPImage *in, MPImage *out,
                             int nimgs, uint64_t seed, uint64_t index0)
{
    if (nimgs < 0 || nstages < 0 || (nimgs > 0 && (!in || !out))) return MP_ERROR_INVALID_ARGS;
    std::vector<ROp> ops;
    std::vector<Seg> segs;
    for (int i = 0; i < nimgs; ++i) {
        if (in[i].channels != 1 && in[i].channels != 3 && in[i].channels != 4)
            return MP_ERROR_BAD_DESCRIPTOR;
        MPStatus st = mp_resolve_image(stages, nstages, seed, index0 + (uint64_t)i, ops, nullptr);
        if (st != MILLIPYDE_SUCCESS) return st;
        mp_segment(ops, in[i].channels, in[i].height, in[i].width, segs);
        const Seg &l = segs.back();
        out[i].height = l.hout;
        out[i].width = l.wout;
        out[i].channels = l.cout;
        out[i].pitch = mp_round16((long long)l.wout * l.cout * 4);
    }
    return MILLIPYDE_SUCCESS;
}

MPStatus mpk_pipeline_run(const MPStage *stages, int nstages, const MPImage *in, MPImage *out,
                          int nimgs, uint64_t seed, uint64_t index0, void *stream)
{
    MPPlan *p = nullptr;
    MPStatus st = mpk_plan_create(stages, nstages, in, out, nimgs, seed, index0, stream, &p);
    if (st != MILLIPYDE_SUCCESS) return st;
    st = mpk_plan_launch(p, stream);
    mpk_plan_destroy(p);
    return st;
}

}  // extern "C"

// Plain per-op path: one launch per stage and image, each stage's result in
// device memory (what the reference's Pipeline did, minus its per-stage host
// sync and per-stage allocation).  Intermediates alternate between two
// buffers allocated once per batch (sized for the largest intermediate), so
// the baseline pays the per-op kernels' memory traffic and launches, not
// allocator calls.
static size_t mp_unfused_inter_bytes(const std::vector<ROp> &ops, const MPImage &in)
{
    size_t need = 0;
    int h = in.height, w = in.width, c = in.channels;
    for (size_t k = 0; k + 1 < ops.size(); ++k) {
        std::vector<ROp> one(1, ops[k]);
        std::vector<Seg> sg;
        mp_segment(one, c, h, w, sg);
        const Seg &g = sg.back();
        h = g.hout;
        w = g.wout;
        c = g.cout;
        need = std::max(need, (size_t)h * mp_round16((long long)w * c * 4));
    }
    return need;
}

static MPStatus mp_run_ops_unfused(const std::vector<ROp> &ops, const MPImage &in, const MPImage &out,
                                   void *const bufs[2], cudaStream_t s)
{
    MPImage cur = in;
    if (ops.empty()) {
        std::vector<Seg> sg;
        mp_segment(ops, in.channels, in.height, in.width, sg);
        return mp_run_segment_single(sg[0], in, out, s);
    }
    for (size_t k = 0; k < ops.size(); ++k) {
        std::vector<ROp> one(1, ops[k]);
        std::vector<Seg> sg;
        mp_segment(one, cur.channels, cur.height, cur.width, sg);
        const Seg &g = sg.back();
        MPImage nx;
        if (k + 1 == ops.size()) {
            nx = out;
        } else {
            nx.height = g.hout;
            nx.width = g.wout;
            nx.channels = g.cout;
            nx.pitch = mp_round16((long long)nx.width * nx.channels * 4);
            nx.data = bufs[k & 1];
        }
        MPStatus st = mp_run_segment_single(g, cur, nx, s);
        if (st != MILLIPYDE_SUCCESS) return st;
        cur = nx;
    }
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpk_pipeline_run_unfused(const MPStage *stages, int nstages, const MPImage *in,
                                             MPImage *out, int nimgs, uint64_t seed,
                                             uint64_t index0, void *stream)
{
    if (nimgs < 0 || nstages < 0 || (nimgs > 0 && (!in || !out))) return MP_ERROR_INVALID_ARGS;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<std::vector<ROp>> all(nimgs);
    size_t need = 0;
    for (int i = 0; i < nimgs; ++i) {
        MPStatus st = mp_resolve_image(stages, nstages, seed, index0 + (uint64_t)i, all[i], nullptr);
        if (st != MILLIPYDE_SUCCESS) return st;
        need = std::max(need, mp_unfused_inter_bytes(all[i], in[i]));
    }
    void *bufs[2] = {nullptr, nullptr};
    MPStatus st = mp_malloc_async(&bufs[0], need, s);
    if (st == MILLIPYDE_SUCCESS) st = mp_malloc_async(&bufs[1], need, s);
    for (int i = 0; i < nimgs && st == MILLIPYDE_SUCCESS; ++i) st = mp_run_ops_unfused(all[i], in[i], out[i], bufs, s);
    mp_free_async(bufs[0], s);
    mp_free_async(bufs[1], s);
    return st;
}

// ---------------------------------------------------------------------------
// Per-op entry points on MPObjData (src/millipyde_image.cpp:530-717).
// ---------------------------------------------------------------------------
#define MP_NPY_FLOAT32 11

// Describes a float32 image object; MP_ERROR_UNSUPPORTED_TYPE for others.
static MPStatus mp_obj_image(const MPObjData *o, MPImage *m)
{
    if (!o) return MP_ERROR_INVALID_ARGS;
    if (o->ndims != 2 && o->ndims != 3) return MP_ERROR_UNSUPPORTED_DIMS;
    if (o->type != MP_NPY_FLOAT32) return MP_ERROR_UNSUPPORTED_TYPE;
    m->height = o->dims[0];
    m->width = o->dims[1];
    m->channels = o->ndims == 3 ? o->dims[2] : 1;
    if (m->channels != 1 && m->channels != 3 && m->channels != 4) return MP_ERROR_UNSUPPORTED_TYPE;
    m->pitch = o->dims[o->ndims];
    m->data = o->device_data;
    if ((long long)m->height * m->width > 0 && !m->data) return MP_ERROR_NULL_DATA;
    return MILLIPYDE_SUCCESS;
}

// Points obj at a new float32 image buffer of the given geometry.
static MPStatus mp_obj_set_image(MPObjData *o, void *data, int h, int w, int c, int pitch)
{
    const int nd = (c == 1) ? 2 : 3;
    int *dims = (int *)malloc(sizeof(int) * 2 * nd);
    if (!dims) return MP_ERROR_OUT_OF_MEMORY;
    dims[0] = h;
    dims[1] = w;
    if (nd == 3) dims[2] = c;
    dims[nd] = pitch;
    dims[nd + 1] = (nd == 3) ? c * 4 : 4;
    if (nd == 3) dims[nd + 2] = 4;
    if (o->device_data && o->device_data != data)
        mp_free_async(o->device_data, (cudaStream_t)o->stream);
    free(o->dims);
    o->dims = dims;
    o->ndims = nd;
    o->device_data = data;
    o->type = MP_NPY_FLOAT32;
    o->nbytes = (size_t)h * pitch;
    return MILLIPYDE_SUCCESS;
}

// Runs one op on an object out of place (new pool buffer, old one freed).
static MPStatus mp_obj_apply(MPObjData *o, int op, double p0, double p1, double p2)
{
    MPImage in;
    MPStatus st = mp_obj_image(o, &in);
    if (st == MP_ERROR_UNSUPPORTED_TYPE) return mp_legacy_apply(o, op, p0, p1, p2);
    if (st != MILLIPYDE_SUCCESS) return st;
    ROp r;
    r.op = op;
    r.p[0] = p0;
    r.p[1] = p1;
    r.p[2] = p2;
    st = mp_check_op(op, r.p);
    if (st != MILLIPYDE_SUCCESS) return st;
    MP_CUDA_TRY(cudaSetDevice(o->mem_loc));
    cudaStream_t s = (cudaStream_t)o->stream;
    std::vector<ROp> ops(1, r);
    std::vector<Seg> sg;
    mp_segment(ops, in.channels, in.height, in.width, sg);
    const Seg &g = sg.back();
    // in-place fast path: channel-agnostic pointwise op on 1- or 3-channel data
    if (g.kind == MPK_POINT && !g.flip && (op == MP_OP_BRIGHTNESS || op == MP_OP_ADJUST_GAMMA) &&
        in.channels != 4) {
        PwList L = g.pro;
        return mp_launch_flat((float *)in.data, o->nbytes / 4, L, s);
    }
    if (g.kind == MPK_POINT && !g.flip && g.pro.n == 0 && g.epi.n == 0)
        return MILLIPYDE_SUCCESS;   // identity (e.g. rgb2grey of a grey image)
    MPImage out;
    out.height = g.hout;
    out.width = g.wout;
    out.channels = g.cout;
    out.pitch = mp_round16((long long)out.width * out.channels * 4);
    void *buf = nullptr;
    st = mp_malloc_async(&buf, (size_t)out.height * out.pitch, s);
    if (st != MILLIPYDE_SUCCESS) return st;
    out.data = buf;
    st = mp_run_segment_single(g, in, out, s);
    if (st != MILLIPYDE_SUCCESS) {
        mp_free_async(buf, s);
        return st;
    }
    return mp_obj_set_image(o, buf, out.height, out.width, out.channels, out.pitch);
}

extern "C" {

MPStatus mpimg_color_to_greyscale(MPObjData *obj_data, void *args)
{
    (void)args;
    return mp_obj_apply(obj_data, MP_OP_RGB2GREY, 0, 0, 0);
}

MPStatus mpimg_transpose(MPObjData *obj_data, void *args)
{
    (void)args;
    return mp_obj_apply(obj_data, MP_OP_TRANSPOSE, 0, 0, 0);
}

MPStatus mpimg_gaussian(MPObjData *obj_data, void *args)
{
    if (!args) return MP_ERROR_INVALID_ARGS;
    return mp_obj_apply(obj_data, MP_OP_GAUSSIAN, ((GaussianArgs *)args)->sigma, 0, 0);
}

MPStatus mpimg_fliplr(MPObjData *obj_data, void *args)
{
    (void)args;
    return mp_obj_apply(obj_data, MP_OP_FLIPLR, 0, 0, 0);
}

MPStatus mpimg_rotate(MPObjData *obj_data, void *args)
{
    if (!args) return MP_ERROR_INVALID_ARGS;
    return mp_obj_apply(obj_data, MP_OP_ROTATE, ((RotateArgs *)args)->angle, 0, 0);
}

MPStatus mpimg_brightness(MPObjData *obj_data, void *args)
{
    if (!args) return MP_ERROR_INVALID_ARGS;
    return mp_obj_apply(obj_data, MP_OP_BRIGHTNESS, ((BrightnessArgs *)args)->delta, 0, 0);
}

MPStatus mpimg_colorize(MPObjData *obj_data, void *args)
{
    if (!args) return MP_ERROR_INVALID_ARGS;
    const ColorizeArgs *a = (const ColorizeArgs *)args;
    return mp_obj_apply(obj_data, MP_OP_COLORIZE, a->r_mult, a->g_mult, a->b_mult);
}

MPStatus mpimg_adjust_gamma(MPObjData *obj_data, void *args)
{
    if (!args) return MP_ERROR_INVALID_ARGS;
    const GammaArgs *a = (const GammaArgs *)args;
    return mp_obj_apply(obj_data, MP_OP_ADJUST_GAMMA, a->gamma, a->gain, 0);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Object-level batches for Pipeline.run and Generator.
// ---------------------------------------------------------------------------
static MPStatus mp_obj_apply_resolved(MPObjData *o, const std::vector<ROp> &ops)
{
    for (const ROp &r : ops) {
        MPStatus st = mp_obj_apply(o, r.op, r.p[0], r.p[1], r.p[2]);
        if (st != MILLIPYDE_SUCCESS) return st;
    }
    return MILLIPYDE_SUCCESS;
}

// One batch over distinct objects.
static MPStatus mp_run_objects_once(const MPStage *stages, int nstages, MPObjData **objs,
                                    const std::vector<int> &idx, uint64_t seed, uint64_t index0,
                                    int fused)
{
    const int n = (int)idx.size();
    if (n == 0) return MILLIPYDE_SUCCESS;
    bool all_float = true;
    std::vector<MPImage> in(n), out(n);
    for (int q = 0; q < n; ++q)
        if (mp_obj_image(objs[idx[q]], &in[q]) != MILLIPYDE_SUCCESS) all_float = false;
    if (!all_float) {
        std::vector<ROp> ops;
        for (int q = 0; q < n; ++q) {
            MPStatus st = mp_resolve_image(stages, nstages, seed, index0 + (uint64_t)idx[q], ops, nullptr);
            if (st != MILLIPYDE_SUCCESS) return st;
            st = mp_obj_apply_resolved(objs[idx[q]], ops);
            if (st != MILLIPYDE_SUCCESS) return st;
        }
        return MILLIPYDE_SUCCESS;
    }
    MPObjData *o0 = objs[idx[0]];
    for (int q = 1; q < n; ++q)
        if (objs[idx[q]]->mem_loc != o0->mem_loc) return MP_ERROR_BAD_DESCRIPTOR;
    MP_CUDA_TRY(cudaSetDevice(o0->mem_loc));
    cudaStream_t s = (cudaStream_t)o0->stream;
    for (int q = 1; q < n; ++q)
        if (objs[idx[q]]->stream != o0->stream) cudaStreamSynchronize((cudaStream_t)objs[idx[q]]->stream);
    // shapes per image (each image's own index for random draws)
    for (int q = 0; q < n; ++q) {
        MPStatus st = mpk_pipeline_shapes(stages, nstages, &in[q], &out[q], 1, seed,
                                          index0 + (uint64_t)idx[q]);
        if (st != MILLIPYDE_SUCCESS) return st;
    }
    MPStatus st = MILLIPYDE_SUCCESS;
    for (int q = 0; q < n && st == MILLIPYDE_SUCCESS; ++q)
        st = mp_malloc_async(&out[q].data, (size_t)out[q].height * out[q].pitch, s);
    if (st == MILLIPYDE_SUCCESS) {
        // images keep their list index for random draws: run per contiguous index run
        bool contiguous = true;
        for (int q = 1; q < n; ++q) contiguous &= idx[q] == idx[q - 1] + 1;
        if (contiguous) {
            st = fused ? mpk_pipeline_run(stages, nstages, in.data(), out.data(), n, seed,
                                          index0 + (uint64_t)idx[0], s)
                       : mpk_pipeline_run_unfused(stages, nstages, in.data(), out.data(), n, seed,
                                                  index0 + (uint64_t)idx[0], s);
        } else {
            for (int q = 0; q < n && st == MILLIPYDE_SUCCESS; ++q)
                st = fused ? mpk_pipeline_run(stages, nstages, &in[q], &out[q], 1, seed,
                                              index0 + (uint64_t)idx[q], s)
                           : mpk_pipeline_run_unfused(stages, nstages, &in[q], &out[q], 1, seed,
                                                      index0 + (uint64_t)idx[q], s);
        }
    }
    if (st != MILLIPYDE_SUCCESS) {
        for (int q = 0; q < n; ++q) mp_free_async(out[q].data, s);
        return st;
    }
    for (int q = 0; q < n; ++q) {
        MPObjData *o = objs[idx[q]];
        o->stream = (void *)s;
        st = mp_obj_set_image(o, out[q].data, out[q].height, out[q].width, out[q].channels,
                              out[q].pitch);
        if (st != MILLIPYDE_SUCCESS) return st;
    }
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpk_pipeline_run_objects(const MPStage *stages, int nstages, MPObjData **objs,
                                             int nobjs, uint64_t seed, uint64_t index0, int fused)
{
    if (nobjs < 0 || (nobjs > 0 && !objs) || nstages < 0) return MP_ERROR_INVALID_ARGS;
    // rounds: the k-th occurrence of each object goes into round k
    std::vector<int> round(nobjs, 0);
    int nrounds = nobjs > 0 ? 1 : 0;
    for (int i = 0; i < nobjs; ++i) {
        if (!objs[i]) return MP_ERROR_INVALID_ARGS;
        for (int j = 0; j < i; ++j)
            if (objs[j] == objs[i]) round[i] = std::max(round[i], round[j] + 1);
        nrounds = std::max(nrounds, round[i] + 1);
    }
    for (int r = 0; r < nrounds; ++r) {
        std::vector<int> idx;
        for (int i = 0; i < nobjs; ++i)
            if (round[i] == r) idx.push_back(i);
        MPStatus st = mp_run_objects_once(stages, nstages, objs, idx, seed, index0, fused);
        if (st != MILLIPYDE_SUCCESS) return st;
    }
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpk_pipeline_produce(const MPStage *stages, int nstages, MPObjData **srcs,
                                         MPObjData **outs, int n, uint64_t seed, uint64_t index0)
{
    if (n < 0 || (n > 0 && (!srcs || !outs))) return MP_ERROR_INVALID_ARGS;
    if (n == 0) return MILLIPYDE_SUCCESS;
    std::vector<MPImage> in(n), out(n);
    bool all_float = true;
    for (int i = 0; i < n; ++i)
        if (mp_obj_image(srcs[i], &in[i]) != MILLIPYDE_SUCCESS) all_float = false;
    if (!all_float) {
        std::vector<ROp> ops;
        for (int i = 0; i < n; ++i) {
            MPObjData *c = mpobj_clone_data(srcs[i], srcs[i]->mem_loc, 0);
            if (!c) return MP_ERROR_CUDA;
            MPStatus st = mp_resolve_image(stages, nstages, seed, index0 + (uint64_t)i, ops, nullptr);
            if (st == MILLIPYDE_SUCCESS) st = mp_obj_apply_resolved(c, ops);
            if (st != MILLIPYDE_SUCCESS) {
                mpobj_dealloc_device_data(c);
                free(c);
                for (int k = 0; k < i; ++k) mpobj_dealloc_device_data(outs[k]);
                return st;
            }
            *outs[i] = *c;
            free(c);
        }
        return MILLIPYDE_SUCCESS;
    }
    const int dev = srcs[0]->mem_loc;
    MP_CUDA_TRY(cudaSetDevice(dev));
    cudaStream_t s = (cudaStream_t)mpdev_get_stream(dev, 0);
    if (!s) return MP_ERROR_NO_DEVICE;
    for (int i = 0; i < n; ++i)
        if (srcs[i]->stream != (void *)s) cudaStreamSynchronize((cudaStream_t)srcs[i]->stream);
    MPStatus st = mpk_pipeline_shapes(stages, nstages, in.data(), out.data(), n, seed, index0);
    if (st != MILLIPYDE_SUCCESS) return st;
    for (int i = 0; i < n && st == MILLIPYDE_SUCCESS; ++i)
        st = mp_malloc_async(&out[i].data, (size_t)out[i].height * out[i].pitch, s);
    if (st == MILLIPYDE_SUCCESS)
        st = mpk_pipeline_run(stages, nstages, in.data(), out.data(), n, seed, index0, s);
    if (st != MILLIPYDE_SUCCESS) {
        for (int i = 0; i < n; ++i) mp_free_async(out[i].data, s);
        return st;
    }
    for (int i = 0; i < n; ++i) {
        MPObjData *o = outs[i];
        memset(o, 0, sizeof(*o));
        o->mem_loc = dev;
        o->stream = (void *)s;
        o->type = MP_NPY_FLOAT32;
        st = mp_obj_set_image(o, out[i].data, out[i].height, out[i].width, out[i].channels,
                              out[i].pitch);
        if (st != MILLIPYDE_SUCCESS) return st;
    }
    return MILLIPYDE_SUCCESS;
}

// ---------------------------------------------------------------------------
// Host-buffer batch with copy/compute overlap.
// ---------------------------------------------------------------------------
#define MP_HOST_CHUNK_BYTES (192ull << 20)
#define MP_HOST_SLOTS 3

static cudaStream_t mp_copy_stream(int dev, int which)
{
    static cudaStream_t streams[64][2];
    static std::mutex mtx;
    std::lock_guard<std::mutex> lk(mtx);
    if (dev < 0 || dev >= 64) return nullptr;
    if (!streams[dev][which]) {
        if (cudaStreamCreateWithFlags(&streams[dev][which], cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            streams[dev][which] = nullptr;
        }
    }
    return streams[dev][which];
}

extern "C" MPStatus mpk_pipeline_run_host(const MPStage *stages, int nstages, const MPImage *in,
                                          const MPImage *out, int n, uint64_t seed, uint64_t index0,
                                          void *stream_v)
{
    if (n < 0 || nstages < 0 || (n > 0 && (!in || !out))) return MP_ERROR_INVALID_ARGS;
    if (n == 0) return MILLIPYDE_SUCCESS;
    int dev = 0;
    MP_CUDA_TRY(cudaGetDevice(&dev));
    cudaStream_t cs = stream_v ? (cudaStream_t)stream_v : (cudaStream_t)mpdev_get_stream(dev, 0);
    cudaStream_t hs = mp_copy_stream(dev, 0), ds = mp_copy_stream(dev, 1);
    if (!cs || !hs || !ds) return MP_ERROR_NO_DEVICE;

    // device geometry and chunks of consecutive images
    std::vector<MPImage> din(n), dout(n);
    std::vector<size_t> in_off(n), out_off(n);
    std::vector<std::pair<int, int>> chunks;
    size_t max_in = 0, max_out = 0;
    {
        size_t cin = 0, cout = 0;
        int first = 0;
        for (int i = 0; i < n; ++i) {
            din[i] = in[i];
            din[i].pitch = mp_round16((long long)in[i].width * in[i].channels * 4);
            MPStatus st = mpk_pipeline_shapes(stages, nstages, &in[i], &dout[i], 1, seed, index0 + (uint64_t)i);
            if (st != MILLIPYDE_SUCCESS) return st;
            if (dout[i].height != out[i].height || dout[i].width != out[i].width ||
                dout[i].channels != out[i].channels ||
                out[i].pitch < out[i].width * out[i].channels * 4 ||
                in[i].pitch < in[i].width * in[i].channels * 4)
                return MP_ERROR_BAD_DESCRIPTOR;
            const size_t bi = (size_t)din[i].height * din[i].pitch;
            const size_t bo = (size_t)dout[i].height * dout[i].pitch;
            if (i > first && cin + bi > MP_HOST_CHUNK_BYTES) {
                chunks.push_back({first, i - first});
                max_in = std::max(max_in, cin);
                max_out = std::max(max_out, cout);
                first = i;
                cin = cout = 0;
            }
            in_off[i] = cin;
            out_off[i] = cout;
            cin += (bi + 255) / 256 * 256;
            cout += (bo + 255) / 256 * 256;
        }
        chunks.push_back({first, n - first});
        max_in = std::max(max_in, cin);
        max_out = std::max(max_out, cout);
    }
    // three slots: the copy of chunk k + 3 waits for chunk k's compute, and
    // chunk k's compute for chunk k - 3's results to leave, so the two link
    // directions and the kernels run with a chunk of slack between them
    // (measured on 1000 ragged images, 8.08 GB over the link: 36.0 ms against
    // 36.2 with two slots; the same copies with no kernels take 34.4 ms, so
    // the link bounds the call)
    const int nslots = (int)std::min<size_t>(MP_HOST_SLOTS, chunks.size());
    void *ibuf[MP_HOST_SLOTS] = {}, *obuf[MP_HOST_SLOTS] = {};
    // Packed landing buffers: an image whose host rows are packed crosses
    // the link as one 1-D copy and is re-pitched on the device (and the
    // reverse for results).  Measured on GB300: 2-D host-to-device copies
    // of 1.5 KB rows ran at 35 GB/s (21 GB/s per 129-row image), of 6.9 KB
    // rows at 107 GB/s, a 1-D copy at 212 GB/s.
    void *lin[MP_HOST_SLOTS] = {}, *lout[MP_HOST_SLOTS] = {};
    std::vector<MPPlan *> plans(chunks.size(), nullptr);
    cudaEvent_t ev[4][MP_HOST_SLOTS] = {};
    bool ev_ok = true;
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < MP_HOST_SLOTS; ++b)
            ev_ok &= cudaEventCreateWithFlags(&ev[a][b], cudaEventDisableTiming) == cudaSuccess;
    enum { E_H2D = 0, E_COMP = 1, E_D2H = 2, E_ALLOC = 3 };
    MPStatus st = ev_ok ? MILLIPYDE_SUCCESS : MP_ERROR_CUDA;
    for (int s = 0; s < nslots && st == MILLIPYDE_SUCCESS; ++s) {
        st = mp_malloc_async(&ibuf[s], max_in, cs);
        if (st == MILLIPYDE_SUCCESS) st = mp_malloc_async(&obuf[s], max_out, cs);
        if (st == MILLIPYDE_SUCCESS) st = mp_malloc_async(&lin[s], max_in, cs);
        if (st == MILLIPYDE_SUCCESS) st = mp_malloc_async(&lout[s], max_out, cs);
    }
    // every plan is created (and its job table uploaded) before any copy is
    // queued, so the host never waits on the compute stream inside the loop.
    // Images whose host rows are packed but whose device pitch differs land
    // packed and are re-pitched by an identity plan (the copy kernel) on the
    // copy stream, in both directions, so the copy engines carry only the
    // link's bytes.
    std::vector<MPPlan *> rin(chunks.size(), nullptr), rout(chunks.size(), nullptr);
    auto land_in = [&](int i) { return (size_t)in[i].pitch == (size_t)in[i].width * in[i].channels * 4 &&
                                       in[i].pitch != din[i].pitch && din[i].height > 0 && din[i].width > 0; };
    auto land_out = [&](int i) { return (size_t)out[i].pitch == (size_t)dout[i].width * dout[i].channels * 4 &&
                                        out[i].pitch != dout[i].pitch && dout[i].height > 0 && dout[i].width > 0; };
    for (size_t k = 0; k < chunks.size() && st == MILLIPYDE_SUCCESS; ++k) {
        const int slot = (int)(k % nslots), f = chunks[k].first, c = chunks[k].second;
        std::vector<MPImage> ls, ld, ms, md;
        for (int i = f; i < f + c; ++i) {
            din[i].data = (char *)ibuf[slot] + in_off[i];
            dout[i].data = (char *)obuf[slot] + out_off[i];
            if (land_in(i)) {
                MPImage l = din[i];
                l.data = (char *)lin[slot] + in_off[i];
                l.pitch = in[i].pitch;
                ls.push_back(l);
                ld.push_back(din[i]);
            }
            if (land_out(i)) {
                MPImage l = dout[i];
                l.data = (char *)lout[slot] + out_off[i];
                l.pitch = out[i].pitch;
                ms.push_back(dout[i]);
                md.push_back(l);
            }
        }
        st = mpk_plan_create(stages, nstages, &din[f], &dout[f], c, seed, index0 + (uint64_t)f, cs,
                             &plans[k]);
        if (st == MILLIPYDE_SUCCESS && !ls.empty())
            st = mpk_plan_create(nullptr, 0, ls.data(), ld.data(), (int)ls.size(), 0, 0, cs, &rin[k]);
        if (st == MILLIPYDE_SUCCESS && !ms.empty())
            st = mpk_plan_create(nullptr, 0, ms.data(), md.data(), (int)ms.size(), 0, 0, cs, &rout[k]);
    }
    if (st == MILLIPYDE_SUCCESS) {
        st = mp_cuda_status(cudaEventRecord(ev[E_ALLOC][0], cs));
        if (st == MILLIPYDE_SUCCESS) cudaStreamWaitEvent(hs, ev[E_ALLOC][0], 0);
        if (st == MILLIPYDE_SUCCESS) cudaStreamWaitEvent(ds, ev[E_ALLOC][0], 0);
    }
    for (size_t k = 0; k < chunks.size() && st == MILLIPYDE_SUCCESS; ++k) {
        const int slot = (int)(k % nslots), f = chunks[k].first, c = chunks[k].second;
        if (k >= (size_t)nslots) cudaStreamWaitEvent(hs, ev[E_COMP][slot], 0);   // input slot free
        for (int i = f; i < f + c && st == MILLIPYDE_SUCCESS; ++i) {
            if (din[i].height <= 0 || din[i].width <= 0) continue;
            const size_t rb = (size_t)in[i].width * in[i].channels * 4, h = (size_t)in[i].height;
            if ((size_t)in[i].pitch == (size_t)din[i].pitch) {
                // same row pitch on both sides: the rows and their padding in one copy
                st = mp_cuda_status(cudaMemcpyAsync(din[i].data, in[i].data, (h - 1) * (size_t)in[i].pitch + rb,
                                                    cudaMemcpyHostToDevice, hs));
            } else if (land_in(i)) {
                st = mp_cuda_status(cudaMemcpyAsync((char *)lin[slot] + in_off[i], in[i].data, h * rb,
                                                    cudaMemcpyHostToDevice, hs));
            } else {
                st = mp_cuda_status(cudaMemcpy2DAsync(din[i].data, din[i].pitch, in[i].data, in[i].pitch, rb, h,
                                                      cudaMemcpyHostToDevice, hs));
            }
        }
        if (st == MILLIPYDE_SUCCESS && rin[k]) st = mpk_plan_launch(rin[k], hs);
        if (st != MILLIPYDE_SUCCESS) break;
        cudaEventRecord(ev[E_H2D][slot], hs);
        cudaStreamWaitEvent(cs, ev[E_H2D][slot], 0);
        if (k >= (size_t)nslots) cudaStreamWaitEvent(cs, ev[E_D2H][slot], 0);   // output slot free
        st = mpk_plan_launch(plans[k], cs);
        if (st != MILLIPYDE_SUCCESS) break;
        cudaEventRecord(ev[E_COMP][slot], cs);
        cudaStreamWaitEvent(ds, ev[E_COMP][slot], 0);
        if (st == MILLIPYDE_SUCCESS && rout[k]) st = mpk_plan_launch(rout[k], ds);
        for (int i = f; i < f + c && st == MILLIPYDE_SUCCESS; ++i) {
            if (dout[i].height <= 0 || dout[i].width <= 0) continue;
            const size_t rb = (size_t)dout[i].width * dout[i].channels * 4, h = (size_t)dout[i].height;
            if (land_out(i)) {
                st = mp_cuda_status(cudaMemcpyAsync(out[i].data, (char *)lout[slot] + out_off[i], h * rb,
                                                    cudaMemcpyDeviceToHost, ds));
            } else {
                st = mp_cuda_status(cudaMemcpy2DAsync(out[i].data, out[i].pitch, dout[i].data, dout[i].pitch, rb, h,
                                                      cudaMemcpyDeviceToHost, ds));
            }
        }
        cudaEventRecord(ev[E_D2H][slot], ds);
    }
    cudaStreamSynchronize(hs);
    cudaStreamSynchronize(ds);
    cudaStreamSynchronize(cs);
    for (MPPlan *p : plans) mpk_plan_destroy(p);
    for (MPPlan *p : rin) mpk_plan_destroy(p);
    for (MPPlan *p : rout) mpk_plan_destroy(p);
    for (int s = 0; s < MP_HOST_SLOTS; ++s) {
        mp_free_async(lin[s], cs);
        mp_free_async(lout[s], cs);
        mp_free_async(ibuf[s], cs);
        mp_free_async(obuf[s], cs);
    }
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < MP_HOST_SLOTS; ++b)
            if (ev[a][b]) cudaEventDestroy(ev[a][b]);
    if (st != MILLIPYDE_SUCCESS) return st;
    return mp_check_device_error(cs);
}

// ---------------------------------------------------------------------------
// Differentiable chains on dense batches (the autograd path).
//   x: B images of H x W x C float32, packed (pitch W*C*4), image b at
//   x + b*H*W*C; ops[nops] op codes; params[(b*nops + k)*3 + j] explicit
//   per-image parameters (angle / sigma / delta / gamma, gain / r, g, b).
// ---------------------------------------------------------------------------
struct MPShape { int h, w, c; };

static MPStatus mp_chain_shapes(const int *ops, int nops, int H, int W, int C,
                                std::vector<MPShape> &sh)
{
    if (nops < 0 || H < 0 || W < 0 || (C != 1 && C != 3 && C != 4)) return MP_ERROR_BAD_DESCRIPTOR;
    sh.assign(nops + 1, MPShape{H, W, C});
    for (int k = 0; k < nops; ++k) {
        MPShape n = sh[k];
        switch (ops[k]) {
        case MP_OP_RGB2GREY: if (n.c >= 3) n.c = 1; break;
        case MP_OP_TRANSPOSE: std::swap(n.h, n.w); break;
        case MP_OP_GAUSSIAN: case MP_OP_FLIPLR: case MP_OP_ROTATE: case MP_OP_BRIGHTNESS:
        case MP_OP_ADJUST_GAMMA: case MP_OP_COLORIZE: break;
        default: return MP_ERROR_BAD_DESCRIPTOR;
        }
        sh[k + 1] = n;
    }
    return MILLIPYDE_SUCCESS;
}

static MPImage mp_dense_image(const float *base, int b, const MPShape &s)
{
    MPImage m;
    m.data = (void *)(base + (size_t)b * s.h * s.w * s.c);
    m.height = s.h;
    m.width = s.w;
    m.channels = s.c;
    m.pitch = s.w * s.c * 4;
    return m;
}

static ROp mp_rop(int op, const double *p)
{
    ROp r;
    r.op = op;
    r.p[0] = p[0];
    r.p[1] = p[1];
    r.p[2] = p[2];
    return r;
}

extern "C" MPStatus mpk_chain_shape(const int *ops, int nops, int H, int W, int C, int *Ho, int *Wo,
                                    int *Co)
{
    std::vector<MPShape> sh;
    MPStatus st = mp_chain_shapes(ops, nops, H, W, C, sh);
    if (st != MILLIPYDE_SUCCESS) return st;
    if (Ho) *Ho = sh.back().h;
    if (Wo) *Wo = sh.back().w;
    if (Co) *Co = sh.back().c;
    return MILLIPYDE_SUCCESS;
}

// Saved forward intermediates of a chain: the inputs a_k of the ops that
// open the forward plan's second and later segments (the intermediates the
// fused forward writes anyway).  Entry s is a_{idx[s]}, B dense images
// (rows of w*c floats) from byte off[s] of the saved block.  Segmentation
// depends on the op kinds and channels only, so any parameters give the
// same layout.
static void mp_chain_saved_layout(const int *ops, int nops, int B, const std::vector<MPShape> &sh,
                                  std::vector<int> &idx, std::vector<size_t> &off, size_t *total)
{
    std::vector<ROp> kinds(nops);
    for (int k = 0; k < nops; ++k) {
        memset(&kinds[k], 0, sizeof(ROp));
        kinds[k].op = ops[k];
    }
    std::vector<Seg> segs;
    mp_segment(kinds, sh[0].c, sh[0].h, sh[0].w, segs);
    idx.clear();
    off.clear();
    size_t t = 0;
    for (size_t q = 1; q < segs.size(); ++q) {
        const int k = segs[q].op0;
        idx.push_back(k);
        off.push_back(t);
        t += (size_t)B * sh[k].h * sh[k].w * sh[k].c * 4;
    }
    *total = t;
}

extern "C" MPStatus mpk_chain_saved_layout(const int *ops, int nops, int B, int H, int W, int C, int *count,
                                           int *op_index, size_t *offset, size_t *bytes)
{
    if (B < 0 || (nops > 0 && !ops) || !count) return MP_ERROR_INVALID_ARGS;
    std::vector<MPShape> sh;
    MPStatus st = mp_chain_shapes(ops, nops, H, W, C, sh);
    if (st != MILLIPYDE_SUCCESS) return st;
    std::vector<int> idx;
    std::vector<size_t> off;
    size_t total = 0;
    mp_chain_saved_layout(ops, nops, B, sh, idx, off, &total);
    *count = (int)idx.size();
    for (size_t i = 0; i < idx.size(); ++i) {
        if (op_index) op_index[i] = idx[i];
        if (offset) offset[i] = off[i];
    }
    if (bytes) *bytes = total;
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpk_chain_forward_saved(const int *ops, int nops, const double *params, const float *x,
                                            float *y, void *saved, int B, int H, int W, int C, void *stream)
{
    if (B < 0 || (B > 0 && (!x || !y || (nops > 0 && (!ops || !params))))) return MP_ERROR_INVALID_ARGS;
    std::vector<MPShape> sh;
    MPStatus st = mp_chain_shapes(ops, nops, H, W, C, sh);
    if (st != MILLIPYDE_SUCCESS || B == 0) return st;
    std::vector<MPImage> in(B), out(B);
    std::vector<std::vector<ROp>> per(B);
    for (int b = 0; b < B; ++b) {
        in[b] = mp_dense_image(x, b, sh[0]);
        out[b] = mp_dense_image(y, b, sh.back());
        for (int k = 0; k < nops; ++k) per[b].push_back(mp_rop(ops[k], params + ((size_t)b * nops + k) * 3));
    }
    MPInterHomes homes;
    if (saved) {
        std::vector<int> idx;
        std::vector<size_t> off;
        size_t total = 0;
        mp_chain_saved_layout(ops, nops, B, sh, idx, off, &total);
        homes.at.assign(B, std::vector<MPImage>(idx.size()));
        for (int b = 0; b < B; ++b)
            for (size_t q = 0; q < idx.size(); ++q)
                homes.at[b][q] = mp_dense_image((const float *)((const char *)saved + off[q]), b, sh[idx[q]]);
    }
    MPPlanImpl P;
    cudaGetDevice(&P.device);
    P.stream = (cudaStream_t)stream;
    st = mp_plan_build(nullptr, 0, in.data(), out.data(), B, 0, 0, P.stream, &P, &per, saved ? &homes : nullptr);
    if (st == MILLIPYDE_SUCCESS) st = mp_plan_launch(&P, P.stream);
    mp_plan_free(&P, P.stream);
    return st;
}

extern "C" MPStatus mpk_chain_forward(const int *ops, int nops, const double *params, const float *x,
                                      float *y, int B, int H, int W, int C, void *stream)
{
    return mpk_chain_forward_saved(ops, nops, params, x, y, nullptr, B, H, W, C, stream);
}

// Derivative of the normalised gaussian taps with respect to sigma:
// w'_k = w_k (k^2 - sum_j w_j j^2) / sigma^3.
static void mp_gauss_taps(double sigma, int r, float *w, float *dw)
{
    double e[MP_MAX_TAPS], sum = 0.0, m2 = 0.0;
    for (int k = -r; k <= r; ++k) {
        e[k + r] = exp(-(double)(k * k) / (2.0 * sigma * sigma));
        sum += e[k + r];
    }
    for (int k = -r; k <= r; ++k) m2 += e[k + r] / sum * (double)(k * k);
    for (int k = -r; k <= r; ++k) {
        const double wk = e[k + r] / sum;
        w[k + r] = (float)wk;
        if (dw) dw[k + r] = (float)(wk * ((double)(k * k) - m2) / (sigma * sigma * sigma));
    }
}

// Rotate adjoint of op k on the footprint-staged kernel: one RADJ launch
// (dx = R^T g, boxes of g around each source tile) and, when theta wants a
// gradient, one RDTH launch (d theta over output tiles, boxes of the
// source).  Returns false, adding nothing, when some image's rows are not
// TMA-legal or a box does not fit (the caller runs the gather kernel);
// errors of the launches it added go to *st.
template <class SegOf, class AImg, class GoImg, class GiImg, class Acc>
static bool mp_rot_adj_fp(MPTables &T, std::vector<MPLaunch> &launches, int nb, SegOf seg_of, AImg a_img,
                          GoImg gout_img, GiImg gin_img, bool want_theta, Acc acc_of, MPStatus *st)
{
    std::vector<MPJob> ja(nb), jt(want_theta ? nb : 0);
    int bufa = 0, buft = 0;
    for (int q = 0; q < nb; ++q) {
        const Seg sg = seg_of(q);
        const MPImage go = gout_img(q), gi = gin_img(q), a = a_img(q);
        if (!mp_rot_ok(sg, go) || (want_theta && !mp_rot_ok(sg, a))) return false;
        if (mp_fill_job_rot(ja[q], sg, go, gi, true) != MILLIPYDE_SUCCESS) return false;
        const double th_r = sg.core_p[0] * MP_DEG2RAD;
        ja[q].cth = (float)cos(th_r);
        ja[q].sth = (float)sin(th_r);
        bufa = std::max(bufa, mp_rot_buf_floats(ja[q]));
        if (want_theta) {
            if (mp_fill_job_rot(jt[q], sg, a, go) != MILLIPYDE_SUCCESS) return false;
            jt[q].cth = ja[q].cth;
            jt[q].sth = ja[q].sth;
            jt[q].aux = (const float *)go.data;
            jt[q].aux_pitch = go.pitch / 4;
            jt[q].dst = nullptr;
            jt[q].acc = acc_of(q);
            buft = std::max(buft, mp_rot_buf_floats(jt[q]));
        }
    }
    const int C = seg_of(0).cin;
    int ga = 0, gt = 0;
    if (!mp_rot_setup(8 * 1 + C, bufa, &ga)) return false;
    if (want_theta && !mp_rot_setup(8 * 2 + C, buft, &gt)) return false;
    size_t nl = launches.size();
    *st = T.add(launches, MPK_RADJ, 8 * 1 + C, mp_ro_smem(bufa), ja, 0.0);
    if (*st == MILLIPYDE_SUCCESS && launches.size() > nl) {
        launches.back().grid = ga;
        launches.back().gauss[0] = bufa;
    }
    if (*st == MILLIPYDE_SUCCESS && want_theta) {
        nl = launches.size();
        *st = T.add(launches, MPK_RDTH, 8 * 2 + C, mp_ro_smem(buft), jt, 0.0);
        if (*st == MILLIPYDE_SUCCESS && launches.size() > nl) {
            launches.back().grid = gt;
            launches.back().gauss[0] = buft;
        }
    }
    return true;
}

#define MP_BWD_SCRATCH_BYTES (2048ull << 20)

extern "C" MPStatus mpk_chain_backward_masked(const int *ops, int nops, const double *params, const float *x,
                                              const float *dy, float *dx, double *dparams, const int *param_mask,
                                              int B, int H, int W, int C, void *stream);

extern "C" MPStatus mpk_chain_backward(const int *ops, int nops, const double *params, const float *x,
                                       const float *dy, float *dx, double *dparams, int B, int H,
                                       int W, int C, void *stream)
{
    return mpk_chain_backward_masked(ops, nops, params, x, dy, dx, dparams, nullptr, B, H, W, C, stream);
}

extern "C" MPStatus mpk_chain_backward_masked(const int *ops, int nops, const double *params, const float *x,
                                              const float *dy, float *dx, double *dparams, const int *param_mask,
                                              int B, int H, int W, int C, void *stream)
{
    return mpk_chain_backward_saved(ops, nops, params, x, nullptr, nullptr, dy, dx, dparams, param_mask, B, H, W,
                                    C, stream);
}

extern "C" MPStatus mpk_chain_backward_saved(const int *ops, int nops, const double *params, const float *x,
                                             const void *saved, const float *y, const float *dy, float *dx,
                                             double *dparams, const int *param_mask, int B, int H, int W, int C,
                                             void *stream)
{
    // param_mask[k] != 0: the parameters of op k want a gradient (null: all ops)
    auto wants = [&](int k) { return dparams && (!param_mask || param_mask[k] != 0); };
    if (B < 0 || (B > 0 && (!x || !dy || !dx || (nops > 0 && (!ops || !params)))))
        return MP_ERROR_INVALID_ARGS;
    std::vector<MPShape> sh;
    MPStatus st = mp_chain_shapes(ops, nops, H, W, C, sh);
    if (st != MILLIPYDE_SUCCESS || B == 0) return st;
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0;
    cudaGetDevice(&dev);
    int *err = mp_device_error_word(dev);
    if (!err) return MP_ERROR_NO_DEVICE;
    for (int b = 0; b < B; ++b)
        for (int k = 0; k < nops; ++k) {
            MPStatus c = mp_check_op(ops[k], params + ((size_t)b * nops + k) * 3);
            if (c != MILLIPYDE_SUCCESS) return c;
        }
    if (nops == 0) {
        return mp_cuda_status(cudaMemcpyAsync(dx, dy, (size_t)B * H * W * C * 4,
                                              cudaMemcpyDeviceToDevice, s));
    }
    // intermediates the forward saved (a_k of the saved layout), if any
    std::vector<long long> saved_off(nops + 1, -1);
    if (saved) {
        std::vector<int> idx;
        std::vector<size_t> off;
        size_t total = 0;
        mp_chain_saved_layout(ops, nops, B, sh, idx, off, &total);
        for (size_t q = 0; q < idx.size(); ++q) saved_off[idx[q]] = (long long)off[q];
    }
    // intermediates the reverse sweep reads: the input of each pointwise
    // run (grouped as the sweep groups them), of a gaussian whose sigma
    // wants a gradient (the d sigma dot passes) and of every rotate (d theta,
    // and the gather adjoint's source geometry); transpose and fliplr read
    // none.
    // A final lone brightness back-propagates from the chain's output y
    // (when given) and reads no intermediate.
    const bool tail_from_y = y && nops >= 1 && ops[nops - 1] == MP_OP_BRIGHTNESS &&
                             (nops == 1 || !mp_is_pointwise(ops[nops - 2]));
    std::vector<char> need(nops + 1, 0);
    for (int k = nops - 1; k >= 0;) {
        int j = k;
        if (mp_is_pointwise(ops[k]))
            while (j > 0 && mp_is_pointwise(ops[j - 1]) && k - (j - 1) < MP_MAX_PW) --j;
        const bool reads = (mp_is_pointwise(ops[k]) && !(tail_from_y && k == nops - 1)) ||
                           ops[k] == MP_OP_ROTATE || (ops[k] == MP_OP_GAUSSIAN && wants(k));
        if (reads) need[j] = 1;
        k = j - 1;
    }
    // recompute a_{k+1} = op_k(a_k) for k in [rc0, rc1): from the last saved
    // (or the input) at or below the first needed intermediate that was not
    // saved, up to the last one; saved intermediates inside the range are
    // read, not recomputed
    int rc0 = 0, rc1 = 0, lo_unsaved = -1;
    for (int k = 1; k < nops; ++k)
        if (need[k] && saved_off[k] < 0) {
            if (lo_unsaved < 0) lo_unsaved = k;
            rc1 = k;
        }
    if (lo_unsaved > 0)
        for (int k = 1; k <= lo_unsaved; ++k)
            if (saved_off[k] >= 0) rc0 = k;
    // scratch per image: the intermediates recomputed here + two gradient buffers
    size_t inter = 0, gmax = 0;
    std::vector<size_t> aoff(nops + 1, 0);
    for (int k = rc0 + 1; k <= rc1; ++k) {
        if (saved_off[k] >= 0) continue;
        aoff[k] = inter;
        inter += (size_t)sh[k].h * sh[k].w * sh[k].c * 4;
    }
    for (int k = 0; k <= nops; ++k) gmax = std::max(gmax, (size_t)sh[k].h * sh[k].w * sh[k].c * 4);
    const size_t per_img = inter + 2 * gmax;
    int chunk = (int)std::max<size_t>(1, MP_BWD_SCRATCH_BYTES / std::max<size_t>(per_img, 1));
    chunk = std::min(chunk, B);
    void *scratch = nullptr;
    st = mp_malloc_async(&scratch, per_img * (size_t)chunk, s);
    if (st != MILLIPYDE_SUCCESS) return st;
    char *sbase = (char *)scratch;
    for (int b0 = 0; b0 < B && st == MILLIPYDE_SUCCESS; b0 += chunk) {
        const int nb = std::min(chunk, B - b0);
        // per-image pointers inside the chunk's scratch
        auto a_img = [&](int q, int k) -> MPImage {       // input of op k for image b0+q
            if (k == 0) return mp_dense_image(x, b0 + q, sh[0]);
            if (saved_off[k] >= 0)
                return mp_dense_image((const float *)((const char *)saved + saved_off[k]), b0 + q, sh[k]);
            MPImage m = mp_dense_image((const float *)(sbase + (size_t)q * per_img + aoff[k]), 0, sh[k]);
            return m;
        };
        auto g_img = [&](int q, int which, const MPShape &shp) -> MPImage {
            return mp_dense_image((const float *)(sbase + (size_t)q * per_img + inter + which * gmax), 0, shp);
        };
        MPPlanImpl P;
        P.device = dev;
        P.stream = s;
        P.err = err;
        MPTables T;
        auto add_launch = [&](int kind, size_t smem, std::vector<MPJob> &js) -> MPStatus {
            int v = 0;
            if ((kind == MPK_GAUSS || kind == MPK_ROTATE) && !js.empty()) v = mp_variant(js[0].cin, js[0].cmid);
            return T.add(P.launches, kind, v, smem, js, 0.0);
        };
        // one-op segment for op k of image q
        auto seg_of = [&](int q, int k) -> Seg {
            std::vector<ROp> one(1, mp_rop(ops[k], params + ((size_t)(b0 + q) * nops + k) * 3));
            std::vector<Seg> sg;
            mp_segment(one, sh[k].c, sh[k].h, sh[k].w, sg);
            return sg.back();
        };
        auto gauss_launch = [&](std::vector<std::pair<Seg, std::pair<MPImage, MPImage>>> &items,
                                std::vector<MPJob> &js, size_t *smem) -> MPStatus {
            int rmax = 1, cm = 1;
            for (auto &it : items) {
                rmax = std::max(rmax, (int)ceil(3.0 * it.first.core_p[0]));
                cm = std::max(cm, it.first.cmid);
            }
            int tw, th;
            mp_gauss_tiles(rmax, cm, cm, 0, &tw, &th);
            *smem = mp_gauss_smem_bytes(tw, th, rmax, cm, cm, 0);
            for (auto &it : items) {
                MPJob J;
                MPStatus e = mp_fill_job(J, it.first, it.second.first, it.second.second, tw, th);
                if (e != MILLIPYDE_SUCCESS) return e;
                js.push_back(J);
            }
            return MILLIPYDE_SUCCESS;
        };
        // ---- forward recompute of the intermediates the adjoints read
        for (int k = rc0; k < rc1 && st == MILLIPYDE_SUCCESS; ++k) {
            if (saved_off[k + 1] >= 0) continue;
            std::vector<MPJob> js;
            size_t smem = 0;
            const int kind = seg_of(0, k).kind;
            if (kind == MPK_GAUSS) {
                std::vector<Seg> sgs;
                std::vector<MPImage> srcs, dsts;
                for (int q = 0; q < nb; ++q) {
                    sgs.push_back(seg_of(q, k));
                    srcs.push_back(a_img(q, k));
                    dsts.push_back(a_img(q, k + 1));
                }
                st = mp_add_gauss(T, P.launches, sgs, srcs, dsts);
                continue;
            } else {
                if (kind == MPK_ROTATE) {
                    std::vector<Seg> sgs;
                    std::vector<MPImage> srcs, dsts;
                    for (int q = 0; q < nb; ++q) {
                        sgs.push_back(seg_of(q, k));
                        srcs.push_back(a_img(q, k));
                        dsts.push_back(a_img(q, k + 1));
                    }
                    bool added = false;
                    st = mp_add_rot(T, P.launches, sgs, srcs, dsts, &added);
                    if (st != MILLIPYDE_SUCCESS || added) continue;
                }
                for (int q = 0; q < nb && st == MILLIPYDE_SUCCESS; ++q) {
                    MPJob J;
                    st = mp_fill_job(J, seg_of(q, k), a_img(q, k), a_img(q, k + 1), 0, 0);
                    js.push_back(J);
                }
            }
            if (st == MILLIPYDE_SUCCESS) st = add_launch(kind, smem, js);
        }
        // ---- reverse sweep
        int cur = -1;   // gradient buffer holding g (output of op k); -1: dy
        int k = nops - 1;
        while (k >= 0 && st == MILLIPYDE_SUCCESS) {
            int j = k;
            const bool pw = mp_is_pointwise(ops[k]);
            if (pw)
                while (j > 0 && mp_is_pointwise(ops[j - 1]) && k - (j - 1) < MP_MAX_PW) --j;
            const int nxt = (j == 0) ? -2 : (cur == 0 ? 1 : 0);   // -2: write dx
            auto gin_img = [&](int q) -> MPImage {
                return nxt == -2 ? mp_dense_image(dx, b0 + q, sh[0]) : g_img(q, nxt, sh[j]);
            };
            auto gout_img = [&](int q) -> MPImage {
                return cur == -1 ? mp_dense_image(dy, b0 + q, sh[nops]) : g_img(q, cur, sh[k + 1]);
            };
            std::vector<MPJob> js;
            if (pw) {
                for (int q = 0; q < nb; ++q) {
                    MPJob J;
                    Seg sg;
                    memset(&sg, 0, sizeof(sg));
                    sg.kind = MPK_POINT;
                    sg.cin = sh[j].c;
                    for (int t = j; t <= k; ++t) {
                        ROp r = mp_rop(ops[t], params + ((size_t)(b0 + q) * nops + t) * 3);
                        mp_pw_push(sg.pro, r);
                    }
                    // the final lone brightness reads the chain's output
                    const bool from_y = tail_from_y && k == nops - 1 && j == k;
                    const MPImage a = from_y ? mp_dense_image(y, b0 + q, sh[nops]) : a_img(q, j);
                    const MPImage go = gout_img(q), gi = gin_img(q);
                    st = mp_fill_job(J, sg, a, gi, 0, 0);
                    if (st != MILLIPYDE_SUCCESS) break;
                    if (from_y) J.pro.op[0].op = MP_OP_BRIGHTNESS_OUT;
                    J.cin = sh[j].c;
                    J.aux = (const float *)go.data;
                    J.aux_pitch = go.pitch / 4;
                    bool any = false;
                    for (int t = j; t <= k; ++t) any = any || wants(t);
                    J.acc = any ? dparams + (size_t)(b0 + q) * nops * 3 : nullptr;
                    for (int t = j; t <= k; ++t) J.pw_slot[t - j] = t;
                    js.push_back(J);
                }
                if (st == MILLIPYDE_SUCCESS) st = add_launch(MPK_POINT_ADJ, 0, js);
            } else if (ops[k] == MP_OP_GAUSSIAN) {
                // dx = blur(g) (the zero-padded gaussian is self-adjoint)
                {
                    std::vector<Seg> sgs;
                    std::vector<MPImage> srcs, dsts;
                    for (int q = 0; q < nb; ++q) {
                        sgs.push_back(seg_of(q, k));
                        srcs.push_back(gout_img(q));
                        dsts.push_back(gin_img(q));
                    }
                    st = mp_add_gauss(T, P.launches, sgs, srcs, dsts);
                }
                size_t smem = 0;
                // d sigma = <g, (W' (x) W + W (x) W') a_k>: two dot-mode launches,
                // only when sigma wants a gradient; the streaming kernels' dot
                // mode when every image can take it (images in radius order),
                // else the tile kernel's
                bool vdot = wants(k) && st == MILLIPYDE_SUCCESS;
                int dcode = -1, dgrid = 0;
                std::vector<int> qord(nb);
                for (int q = 0; q < nb; ++q) qord[q] = q;
                long long drows = 0;
                for (int q = 0; q < nb && vdot; ++q) {
                    const Seg sg = seg_of(q, k);
                    const int r = (int)ceil(3.0 * sg.core_p[0]);
                    const int c = mp_vh_dot_code(sg.cin, r);
                    vdot = c >= 0 && (dcode < 0 || c == dcode) && mp_vh_ok(sg, a_img(q, k));
                    dcode = c;
                    const int cm = (c & 15) > 4 ? sg.cin : 1;
                    const int sw = mp_vh_fit_strip(r, sh[k].w, cm);
                    drows += (long long)((sh[k].w * cm + sw - 1) / sw) * sh[k].h;
                }
                int dcps = 0;
                if (vdot && mp_vh_prepare(dcode, &dcps) != MILLIPYDE_SUCCESS) {
                    cudaGetLastError();
                    vdot = false;
                }
                if (vdot) {
                    dgrid = dcps * mp_num_sms();
                    std::stable_sort(qord.begin(), qord.end(), [&](int a, int b) {
                        return seg_of(a, k).core_p[0] < seg_of(b, k).core_p[0];
                    });
                    const int rs = mp_vh_rows(drows, dgrid);
                    for (int pass = 0; pass < 2 && st == MILLIPYDE_SUCCESS; ++pass) {
                        std::vector<MPJob> jd(nb);
                        for (int i = 0; i < nb && st == MILLIPYDE_SUCCESS; ++i) {
                            const int q = qord[i];
                            const Seg sg = seg_of(q, k);
                            const MPImage go = gout_img(q);
                            MPJob &J = jd[i];
                            st = mp_fill_job_vh(J, sg, a_img(q, k), go, rs);
                            if (st != MILLIPYDE_SUCCESS) break;
                            float w[MP_MAX_TAPS], dw[MP_MAX_TAPS];
                            mp_gauss_taps(sg.core_p[0], J.radius, w, dw);
                            for (int t = 0; t < 2 * J.radius + 1; ++t) {
                                J.wts[t] = pass == 0 ? dw[t] : w[t];
                                J.wts_h[t] = pass == 0 ? w[t] : dw[t];
                            }
                            J.dot = 1;
                            J.aux = (const float *)go.data;
                            J.aux_pitch = go.pitch / 4;
                            J.dst = nullptr;
                            J.acc = dparams + ((size_t)(b0 + q) * nops + k) * 3;
                        }
                        if (st != MILLIPYDE_SUCCESS) break;
                        const size_t nl = P.launches.size();
                        st = T.add(P.launches, MPK_VH, dcode, 0, jd, 0.0);
                        if (st == MILLIPYDE_SUCCESS && P.launches.size() > nl) P.launches.back().grid = dgrid;
                    }
                }
                for (int pass = 0; pass < 2 && wants(k) && !vdot && st == MILLIPYDE_SUCCESS; ++pass) {
                    std::vector<std::pair<Seg, std::pair<MPImage, MPImage>>> it2;
                    for (int q = 0; q < nb; ++q) it2.push_back({seg_of(q, k), {a_img(q, k), gout_img(q)}});
                    std::vector<MPJob> jd;
                    st = gauss_launch(it2, jd, &smem);
                    for (int q = 0; q < nb && st == MILLIPYDE_SUCCESS; ++q) {
                        MPJob &J = jd[q];
                        float w[MP_MAX_TAPS], dw[MP_MAX_TAPS];
                        mp_gauss_taps(it2[q].first.core_p[0], J.radius, w, dw);
                        for (int t = 0; t < 2 * J.radius + 1; ++t) {
                            J.wts[t] = pass == 0 ? dw[t] : w[t];
                            J.wts_h[t] = pass == 0 ? w[t] : dw[t];
                        }
                        J.hsep = 1;
                        J.dot = 1;
                        const MPImage go = gout_img(q);
                        J.aux = (const float *)go.data;
                        J.aux_pitch = go.pitch / 4;
                        J.dst = nullptr;
                        J.acc = dparams + ((size_t)(b0 + q) * nops + k) * 3;
                    }
                    if (st == MILLIPYDE_SUCCESS) st = add_launch(MPK_GAUSS, smem, jd);
                }
            } else if (ops[k] == MP_OP_ROTATE &&
                       mp_rot_adj_fp(
                           T, P.launches, nb, [&](int q) { return seg_of(q, k); },
                           [&](int q) { return a_img(q, k); }, gout_img, gin_img, wants(k),
                           [&](int q) { return dparams + ((size_t)(b0 + q) * nops + k) * 3; }, &st)) {
                // dx = R^T g and d theta on the footprint-staged kernel
            } else if (ops[k] == MP_OP_ROTATE) {
                for (int q = 0; q < nb && st == MILLIPYDE_SUCCESS; ++q) {
                    MPJob J;
                    const Seg sg = seg_of(q, k);
                    const MPImage a = a_img(q, k), go = gout_img(q), gi = gin_img(q);
                    st = mp_fill_job(J, sg, a, gi, 0, 0);
                    const double th_r = sg.core_p[0] * MP_DEG2RAD;
                    J.cth = (float)cos(th_r);
                    J.sth = (float)sin(th_r);
                    J.aux = (const float *)go.data;
                    J.aux_pitch = go.pitch / 4;
                    J.acc = wants(k) ? dparams + ((size_t)(b0 + q) * nops + k) * 3 : nullptr;
                    js.push_back(J);
                }
                if (st == MILLIPYDE_SUCCESS) st = add_launch(MPK_ROTATE_ADJ, 0, js);
            } else {
                // transpose / fliplr: the adjoint is the same permutation of g
                for (int q = 0; q < nb && st == MILLIPYDE_SUCCESS; ++q) {
                    MPJob J;
                    const Seg sg = seg_of(q, k);
                    const MPImage go = gout_img(q), gi = gin_img(q);
                    Seg g2 = sg;
                    if (ops[k] == MP_OP_TRANSPOSE) {
                        g2.hin = sh[k + 1].h;
                        g2.win = sh[k + 1].w;
                    }
                    st = mp_fill_job(J, g2, go, gi, 0, 0);
                    js.push_back(J);
                }
                if (st == MILLIPYDE_SUCCESS) st = add_launch(ops[k] == MP_OP_TRANSPOSE ? MPK_TRANSPOSE : MPK_POINT, 0, js);
            }
            cur = nxt;
            k = j - 1;
        }
        if (st == MILLIPYDE_SUCCESS) st = mp_plan_finish(&P, T, s);
        if (st == MILLIPYDE_SUCCESS) st = mp_plan_launch(&P, s);
        mp_plan_free(&P, s);
    }
    mp_free_async(scratch, s);
    return st;
}

// ---------------------------------------------------------------------------
// One image through its segments with caller-provided intermediate buffers
// (used by the allocation-free entry point in mp_noalloc.cu).
// ---------------------------------------------------------------------------
MPStatus mp_run_image_noalloc(const MPStage *stages, int nstages, uint64_t seed, uint64_t index,
                              const MPImage &in, const MPImage &out, void *half0, void *half1,
                              size_t half_bytes, int *err, cudaStream_t s, bool launch)
{
    if (in.channels != 1 && in.channels != 3 && in.channels != 4) return MP_ERROR_BAD_DESCRIPTOR;
    if (in.height < 0 || in.width < 0 || (in.pitch % 4) ||
        ((long long)in.width * in.channels * 4 > in.pitch && in.height > 0))
        return MP_ERROR_BAD_DESCRIPTOR;
    std::vector<ROp> ops;
    MPStatus st = mp_resolve_image(stages, nstages, seed, index, ops, nullptr);
    if (st != MILLIPYDE_SUCCESS) return st;
    std::vector<Seg> segs;
    mp_segment(ops, in.channels, in.height, in.width, segs);
    const Seg &last = segs.back();
    if (out.height != last.hout || out.width != last.wout || out.channels != last.cout ||
        out.pitch < last.wout * last.cout * 4 || (out.pitch % 4) ||
        (!out.data && (long long)last.hout * last.wout > 0))
        return MP_ERROR_BAD_DESCRIPTOR;
    // every intermediate must fit its half before anything is launched
    for (size_t k = 0; k + 1 < segs.size(); ++k) {
        const size_t need = (size_t)segs[k].hout * mp_round16((long long)segs[k].wout * segs[k].cout * 4);
        if (need > half_bytes) return MP_ERROR_TOO_LARGE;
    }
    if (!launch) return MILLIPYDE_SUCCESS;
    MPImage cur = in;
    for (size_t k = 0; k < segs.size(); ++k) {
        MPImage dst;
        if (k + 1 == segs.size()) {
            dst = out;
        } else {
            dst.height = segs[k].hout;
            dst.width = segs[k].wout;
            dst.channels = segs[k].cout;
            dst.pitch = mp_round16((long long)dst.width * dst.channels * 4);
            dst.data = (k % 2 == 0) ? half0 : half1;
        }
        int tw, th;
        mp_seg_tiles(segs[k], &tw, &th);
        MPJob J;
        st = mp_fill_job(J, segs[k], cur, dst, tw, th);
        if (st != MILLIPYDE_SUCCESS) return st;
        st = mp_launch_single_err(segs[k].kind, J, mp_seg_smem(segs[k], tw, th), err, s);
        if (st != MILLIPYDE_SUCCESS) return st;
        cur = dst;
    }
    return MILLIPYDE_SUCCESS;
}

// ---------------------------------------------------------------------------
// Autotuning hooks
// ---------------------------------------------------------------------------
extern "C" MPStatus mpk_tune_set_gauss_tile(int cin, int cmid, int has_pro, int radius_lo,
                                            int radius_hi, int tw, int th)
{
    if (mp_variant(cin, cmid) < 0 || radius_lo < 1 || radius_hi < radius_lo ||
        radius_hi > MP_MAX_RADIUS)
        return MP_ERROR_INVALID_ARGS;
    if (!mp_gauss_tile_fits(tw, th, radius_hi, cin, cmid, has_pro)) return MP_ERROR_TOO_LARGE;
    std::lock_guard<std::mutex> lk(mp_tune_mutex);
    MPTuneEntry e = {cin, cmid, has_pro ? 1 : 0, radius_lo, radius_hi, tw, th};
    for (MPTuneEntry &x : mp_tune_table)
        if (x.cin == cin && x.cmid == cmid && x.has_pro == e.has_pro && x.rlo == radius_lo &&
            x.rhi == radius_hi) {
            x = e;
            return MILLIPYDE_SUCCESS;
        }
    mp_tune_table.insert(mp_tune_table.begin(), e);
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpk_tune_get_gauss_tile(int cin, int cmid, int has_pro, int radius, int *tw, int *th)
{
    if (mp_variant(cin, cmid) < 0 || radius < 1 || radius > MP_MAX_RADIUS || !tw || !th)
        return MP_ERROR_INVALID_ARGS;
    mp_gauss_tiles(radius, cin, cmid, has_pro, tw, th);
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpk_tune_set_stream(int cmid, int stages)
{
    if ((cmid != 1 && cmid != 3 && cmid != 4) || stages < 2 || stages > MP_GS_MAXNS)
        return MP_ERROR_INVALID_ARGS;
    std::lock_guard<std::mutex> lk(mp_tune_mutex);
    for (MPStreamTune &t : mp_stream_tune)
        if (t.cmid == cmid) {
            t.ns = stages;
            return MILLIPYDE_SUCCESS;
        }
    mp_stream_tune.push_back({cmid, stages});
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpk_tune_set_chunk_bytes(size_t bytes)
{
    if (bytes < ((size_t)1 << 20)) return MP_ERROR_INVALID_ARGS;
    std::lock_guard<std::mutex> lk(mp_tune_mutex);
    mp_chunk_bytes = bytes;
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpk_tune_set_kernel(int kind, int param, int value)
{
    if ((kind != MPK_RSTREAM && kind != MPK_VH && kind != MPK_FUSE) || param < 0 || param >= MP_TK_NPARAM ||
        value < 0)
        return MP_ERROR_INVALID_ARGS;
    if (param == MP_TK_ITEMS && (kind != MPK_VH || value > 64)) return MP_ERROR_INVALID_ARGS;
    if (param == MP_TK_CTAS && value > 32) return MP_ERROR_INVALID_ARGS;
    if (param == MP_TK_STRIP) {
        if (kind != MPK_VH || (value && (value < 64 || value % 8))) return MP_ERROR_INVALID_ARGS;
        mp_vh_set_strip_cap(value);
    }
    std::lock_guard<std::mutex> lk(mp_ktune_mutex);
    mp_ktune[kind][param] = value;
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpk_tune_get_kernel(int kind, int param, int *value)
{
    if (kind < 0 || kind > 15 || param < 0 || param >= MP_TK_NPARAM || !value) return MP_ERROR_INVALID_ARGS;
    *value = mp_tuned(kind, param);
    return MILLIPYDE_SUCCESS;
}

extern "C" MPStatus mpk_tune_set_fuse(int enable)
{
    if (enable != 0 && enable != 1) return MP_ERROR_INVALID_ARGS;
    mp_fuse_mode = enable;
    return MILLIPYDE_SUCCESS;
}

extern "C" void mpk_tune_clear(void)
{
    {
        std::lock_guard<std::mutex> lk(mp_ktune_mutex);
        memset(mp_ktune, 0, sizeof(mp_ktune));
    }
    mp_vh_set_strip_cap(0);
    mp_fuse_mode = 0;
    std::lock_guard<std::mutex> lk(mp_tune_mutex);
    mp_tune_table.clear();
    mp_stream_tune.clear();
}
