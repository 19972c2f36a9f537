// mp_grad.cu -- adjoint kernels of the differentiable path.
//
//   POINT_ADJ   one pass over a run of pointwise ops (rgb2grey, brightness,
//               adjust_gamma, colorize): recomputes the forward values of the
//               run in registers from its input x, back-propagates the
//               output gradient g through the run in reverse and accumulates
//               the parameter gradients (d delta, d gamma, d gain, d mult).
//               A chain's final lone brightness runs from the chain's output
//               instead (MP_OP_BRIGHTNESS_OUT), so its input is not needed.
//   ROTATE_ADJ  dx = R^T g, the exact transpose of the forward bilinear
//               gather: for each source pixel q the kernel visits the (at most
//               4x4) output pixels p whose forward sample used q, recomputes
//               their fixed-point sample position exactly as the forward does
//               and applies the forward's own weight.  No atomics, so dx is
//               deterministic.  The same tile also accumulates
//               d theta = sum_p g(p) . d/dtheta bilinear(x, s(p)).
// The gaussian's adjoint needs no kernel of its own: the zero-padded
// gaussian is self-adjoint (dx = blur(g), a forward GAUSS job), and
// d sigma = <g, (W'(x)W + W(x)W') x> is two GAUSS jobs in dot mode with
// derivative taps (mp_kernels.cu).
//
// Conventions at the kinks (matching the FP64 oracle and the torch-composed
// reference of the tests): a clamp passes gradient only strictly inside
// (0, 1); d/dx x^gamma and d/dgamma are 0 at x = 0.
#include "mp_internal.cuh"

#define MP_THREADS 256
#define MP_DEG2RAD_F 0.01745329252f

__device__ __forceinline__ float mp_block_sum(float v, float *red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    float t = 0.f;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    return t;   // valid in thread 0
}

// Back-propagates g (channels of the op's output) through op `o` whose input
// was v (c channels).  Writes the input gradient to gi, adds parameter
// gradients to pa[0..2].
__device__ __forceinline__ void mp_pw_back(const PwOp &o, const float v[4], int c, const float g[4],
                                           float gi[4], float pa[3])
{
    const int cc = (c == 4) ? 3 : c;
#pragma unroll
    for (int k = 0; k < 4; ++k) gi[k] = g[k];
    switch (o.op) {
    case MP_OP_RGB2GREY: {
        if (c < 3) break;
        const float s = 0.2125f * v[0] + 0.7154f * v[1] + 0.0721f * v[2];
        const float gg = (s < 1.0f) ? g[0] : 0.0f;
        gi[0] = 0.2125f * gg;
        gi[1] = 0.7154f * gg;
        gi[2] = 0.0721f * gg;
        gi[3] = 0.0f;
        break;
    }
    case MP_OP_BRIGHTNESS:
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (k < cc) {
                const float t = v[k] + o.p0;
                const float m = (t > 0.0f && t < 1.0f) ? g[k] : 0.0f;
                gi[k] = m;
                pa[0] += m;
            }
        }
        break;
    case MP_OP_BRIGHTNESS_OUT:
        // v is the op's output: inside (0, 1) iff the clamp was not active
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (k < cc) {
                const float m = (v[k] > 0.0f && v[k] < 1.0f) ? g[k] : 0.0f;
                gi[k] = m;
                pa[0] += m;
            }
        }
        break;
    case MP_OP_ADJUST_GAMMA:
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (k < cc) {
                const float x = v[k];
                float d = 0.0f;
                if (x > 0.0f) {
                    const float pw = __powf(x, o.p0);
                    const float t = o.p1 * pw;
                    if (t > 0.0f && t < 1.0f) {
                        d = g[k] * o.p0 * t / x;
                        pa[0] += g[k] * t * __logf(x);
                        pa[1] += g[k] * pw;
                    }
                }
                gi[k] = d;
            }
        }
        break;
    case MP_OP_COLORIZE:
        if (c < 3) break;
        {
            const float m[3] = {o.p0, o.p1, o.p2};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const bool in = v[k] * m[k] < 1.0f;
                gi[k] = in ? g[k] * m[k] : 0.0f;
                pa[k] += in ? g[k] * v[k] : 0.0f;
            }
        }
        break;
    default:
        break;
    }
}

// One 256 x 4 tile of a pointwise run of NS ops (NS = 0: the run's length
// is read from the job).  For op k from last to first, its input is
// recomputed from x through ops 0..k-1 (runs are short), then g is pulled
// back through op k.  Runs of 1 to 3 ops (nearly all) are compiled with the
// op loops unrolled and one accumulator set per op; longer runs walk the ops
// with loops that are not unrolled.
template <int NS>
__device__ void mp_point_adj_tile(const MPJob &J, int t, float *red)
{
    constexpr int NP = NS ? NS : MP_MAX_PW;   // accumulator sets
    const int ty = t / J.tiles_x, tx = t - ty * J.tiles_x;
    const int x = tx * 256 + threadIdx.x;
    const int n = NS ? NS : J.pro.n, cin = J.cin;
    PwOp ops[NS ? NS : 1];
    if constexpr (NS > 0) {
#pragma unroll
        for (int k = 0; k < NS; ++k) ops[k] = J.pro.op[k];
    }
    auto op_at = [&](int k) -> PwOp { if constexpr (NS > 0) return ops[k]; else return J.pro.op[k]; };
    int cout = cin;
    for (int k = 0; k < n; ++k)
        if (op_at(k).op == MP_OP_RGB2GREY && cout >= 3) cout = 1;
    float pacc[NP][3];
#pragma unroll
    for (int k = 0; k < NP; ++k) pacc[k][0] = pacc[k][1] = pacc[k][2] = 0.f;
    if (x < J.w) {
        // the tile's 4 rows are loaded before any is processed (their loads
        // overlap instead of waiting on each row's compute)
        float x0[4][4], g0[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int y = min(ty * 4 + i, J.h - 1);
            const float *p = J.src + (size_t)y * J.src_pitch + (size_t)x * cin;
            const float *gp = J.aux + (size_t)y * J.aux_pitch + (size_t)x * cout;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                x0[i][c] = (c < cin) ? __ldg(p + c) : 0.f;
                g0[i][c] = (c < cout) ? __ldg(gp + c) : 0.f;
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int y = ty * 4 + i;
            if (y >= J.h) break;
            float g[4] = {g0[i][0], g0[i][1], g0[i][2], g0[i][3]};
            if constexpr (NS > 0) {
#pragma unroll
                for (int k = NS - 1; k >= 0; --k) {
                    float v[4] = {x0[i][0], x0[i][1], x0[i][2], x0[i][3]};
                    int c = cin;
#pragma unroll
                    for (int j = 0; j < k; ++j) c = mp_pw_op(ops[j].op, ops[j].p0, ops[j].p1, ops[j].p2, v, c);
                    float gi[4], pa[3] = {0.f, 0.f, 0.f};
                    mp_pw_back(ops[k], v, c, g, gi, pa);
#pragma unroll
                    for (int q = 0; q < 4; ++q) g[q] = gi[q];
                    pacc[k][0] += pa[0];
                    pacc[k][1] += pa[1];
                    pacc[k][2] += pa[2];
                }
            } else {
#pragma unroll 1
                for (int k = n - 1; k >= 0; --k) {
                    float v[4] = {x0[i][0], x0[i][1], x0[i][2], x0[i][3]};
                    int c = cin;
#pragma unroll 1
                    for (int j = 0; j < k; ++j) {
                        const PwOp o = J.pro.op[j];
                        c = mp_pw_op(o.op, o.p0, o.p1, o.p2, v, c);
                    }
                    float gi[4], pa[3] = {0.f, 0.f, 0.f};
                    mp_pw_back(J.pro.op[k], v, c, g, gi, pa);
#pragma unroll
                    for (int q = 0; q < 4; ++q) g[q] = gi[q];
#pragma unroll
                    for (int kk = 0; kk < MP_MAX_PW; ++kk)
                        if (kk == k) {
                            pacc[kk][0] += pa[0];
                            pacc[kk][1] += pa[1];
                            pacc[kk][2] += pa[2];
                        }
                }
            }
            float *d = J.dst + (size_t)y * J.dst_pitch + (size_t)x * cin;
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (c < cin) d[c] = g[c];
        }
    }
    if (!J.acc) return;
    for (int k = 0; k < n; ++k) {
        const int op = op_at(k).op;
        const int np = (op == MP_OP_BRIGHTNESS || op == MP_OP_BRIGHTNESS_OUT) ? 1
                     : (op == MP_OP_ADJUST_GAMMA) ? 2
                     : (op == MP_OP_COLORIZE) ? 3 : 0;
        for (int j = 0; j < np; ++j) {
            float val = 0.f;
#pragma unroll
            for (int kk = 0; kk < NP; ++kk)
#pragma unroll
                for (int jj = 0; jj < 3; ++jj)
                    if (kk == k && jj == j) val = pacc[kk][jj];
            const float tot = mp_block_sum(val, red);
            if (threadIdx.x == 0) atomicAdd(J.acc + J.pw_slot[k] * 3 + j, (double)tot);
        }
    }
}

// Forward sample position of output pixel (x, y) in MP_FIX_FRAC fixed point,
// bit-identical to the forward ROTATE kernel.
__device__ __forceinline__ void mp_rot_src(const MPJob &J, int x, int y, long long &sx, long long &sy)
{
    const long long W = J.w, H = J.h;
    const long long X2 = 2LL * x - W, Y2 = 2LL * y - H;
    sx = J.cosq * X2 - J.sinq * Y2 + (W << (MP_FIX_FRAC - 1));
    sy = J.sinq * X2 + J.cosq * Y2 + (H << (MP_FIX_FRAC - 1));
}

__device__ __forceinline__ float mp_frac24(long long s)
{
    return (float)((int)((s >> (MP_FIX_FRAC - 24)) & 0xFFFFFF)) * 5.9604644775390625e-8f;
}

__device__ void mp_rotate_adj_tile(const MPJob &J, int t, float *red)
{
    const int ty = t / J.tiles_x, tx = t - ty * J.tiles_x;
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    const int C = J.cin;
    const float hw = 0.5f * (float)J.w, hh = 0.5f * (float)J.h;
    float dth = 0.f;
    for (int i = 0; i < 4; ++i) {
        const int qx = tx * 32 + lx, qy = ty * 32 + ly + 8 * i;
        if (qx >= J.w || qy >= J.h) continue;
        // ---- dx(q): transpose of the forward gather
        const float dxq = (float)qx - hw, dyq = (float)qy - hh;
        const float pxf = J.cth * dxq + J.sth * dyq + hw;     // R(-theta)(q - c) + c
        const float pyf = -J.sth * dxq + J.cth * dyq + hh;
        const int px0 = (int)floorf(pxf) - 1, py0 = (int)floorf(pyf) - 1;
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        // sample positions of the 4 x 4 candidates: the map is affine, so
        // they step exactly by 2 cos / 2 sin from the first one
        long long sxr, syr;
        mp_rot_src(J, px0, py0, sxr, syr);
        const long long c2 = 2 * J.cosq, s2 = 2 * J.sinq;
#pragma unroll
        for (int jy = 0; jy < 4; ++jy) {
            const int py = py0 + jy;
            const bool yok = py >= 0 && py < J.h;
            long long sx = sxr, sy = syr;
#pragma unroll
            for (int jx = 0; jx < 4; ++jx) {
                const int px = px0 + jx;
                const int ix = (int)(sx >> MP_FIX_FRAC), iy = (int)(sy >> MP_FIX_FRAC);
                const int ex = qx - ix, ey = qy - iy;
                if (yok && px >= 0 && px < J.w && (unsigned)ex <= 1u && (unsigned)ey <= 1u) {
                    const float fx = mp_frac24(sx), fy = mp_frac24(sy);
                    const float wx = ex ? fx : 1.0f - fx;
                    const float wy = ey ? fy : 1.0f - fy;
                    const float w = wy * wx;
                    const float *gp = J.aux + (size_t)py * J.aux_pitch + (size_t)px * C;
#pragma unroll
                    for (int c = 0; c < 4; ++c)
                        if (c < C) acc[c] = fmaf(w, __ldg(gp + c), acc[c]);
                }
                sx += c2;
                sy += s2;
            }
            sxr -= s2;
            syr += c2;
        }
        float *d = J.dst + (size_t)qy * J.dst_pitch + (size_t)qx * C;
#pragma unroll
        for (int c = 0; c < 4; ++c)
            if (c < C) d[c] = acc[c];
        // ---- d theta contribution of output pixel p = q
        if (J.acc) {
            long long sx, sy;
            mp_rot_src(J, qx, qy, sx, sy);
            const int ix = (int)(sx >> MP_FIX_FRAC), iy = (int)(sy >> MP_FIX_FRAC);
            const float fx = mp_frac24(sx), fy = mp_frac24(sy);
            const float gx = 1.f - fx, gy = 1.f - fy;
            const float dsx = (-J.sth * dxq - J.cth * dyq) * MP_DEG2RAD_F;
            const float dsy = (J.cth * dxq - J.sth * dyq) * MP_DEG2RAD_F;
            const float *gp = J.aux + (size_t)qy * J.aux_pitch + (size_t)qx * C;
            for (int c = 0; c < C; ++c) {
                float a = 0.f, b = 0.f, cc = 0.f, dd = 0.f;
                const bool x0 = ix >= 0 && ix < J.w, x1 = ix + 1 >= 0 && ix + 1 < J.w;
                const bool y0 = iy >= 0 && iy < J.h, y1 = iy + 1 >= 0 && iy + 1 < J.h;
                const float *s0 = J.src + (size_t)iy * J.src_pitch + c;
                const float *s1 = s0 + J.src_pitch;
                if (y0 && x0) a = __ldg(s0 + (size_t)ix * C);
                if (y0 && x1) b = __ldg(s0 + (size_t)(ix + 1) * C);
                if (y1 && x0) cc = __ldg(s1 + (size_t)ix * C);
                if (y1 && x1) dd = __ldg(s1 + (size_t)(ix + 1) * C);
                const float dvx = gy * (b - a) + fy * (dd - cc);
                const float dvy = gx * (cc - a) + fx * (dd - b);
                dth = fmaf(__ldg(gp + c), dvx * dsx + dvy * dsy, dth);
            }
        }
    }
    if (J.acc) {
        const float tot = mp_block_sum(dth, red);
        if (threadIdx.x == 0) atomicAdd(J.acc, (double)tot);
    }
}

__global__ void __launch_bounds__(MP_THREADS) mp_point_adjoint_batch(const MPJob *__restrict__ jobs,
                                                                     const int *__restrict__ tile_job,
                                                                     int *err)
{
    __shared__ float red[32];
    const int t = blockIdx.x;
    const MPJob &J = jobs[__ldg(tile_job + t)];
    switch (J.pro.n) {
    case 1: mp_point_adj_tile<1>(J, t - J.tile0, red); break;
    case 2: mp_point_adj_tile<2>(J, t - J.tile0, red); break;
    case 3: mp_point_adj_tile<3>(J, t - J.tile0, red); break;
    default: mp_point_adj_tile<0>(J, t - J.tile0, red); break;
    }
}

__global__ void __launch_bounds__(MP_THREADS) mp_rotate_adjoint_batch(const MPJob *__restrict__ jobs,
                                                                      const int *__restrict__ tile_job,
                                                                      int *err)
{
    __shared__ float red[32];
    const int t = blockIdx.x;
    const MPJob &J = jobs[__ldg(tile_job + t)];
    mp_rotate_adj_tile(J, t - J.tile0, red);
}

MPStatus mp_launch_adjoint(int kind, const MPJob *jobs_dev, const int *tile_job, int total_tiles,
                           int *err, cudaStream_t s)
{
    if (total_tiles <= 0) return MILLIPYDE_SUCCESS;
    const void *fn = kind == MPK_ROTATE_ADJ ? (const void *)mp_rotate_adjoint_batch
                                            : (const void *)mp_point_adjoint_batch;
    void *args[] = {(void *)&jobs_dev, (void *)&tile_job, (void *)&err};
    return mp_cuda_status(cudaLaunchKernel(fn, dim3(total_tiles), dim3(MP_THREADS), args, 0, s));
}
