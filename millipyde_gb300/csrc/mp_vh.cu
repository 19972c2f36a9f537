// mp_vh.cu -- host side of the streaming gaussian of mp_vh.cuh: the
// single-channel family (kernels in mp_vh_c1.cu, mp_vh_c3.cu, mp_vh_c4.cu),
// the channel-preserving family (mp_vc_c3.cu, mp_vc_c4.cu) and the
// radius buckets above 12 of the channel-keeping kernels (mp_vb_c*.cu).
#include <mutex>
#include <utility>
#include <vector>

#include "mp_vh.cuh"

#define MP_VH_DECL(NAME)                                                                             \
    __global__ void NAME##_batch(const MPJob *__restrict__, const int *__restrict__, int, int *, int *); \
    __global__ void NAME##_single(const MPJob, int *);
MP_VH_DECL(mp_vh_c1)
MP_VH_DECL(mp_vh_c3)
MP_VH_DECL(mp_vh_c4)
MP_VH_DECL(mp_vc_c3)
MP_VH_DECL(mp_vc_c3_lo)
MP_VH_DECL(mp_vc_c3_mid)
MP_VH_DECL(mp_vc_c4)
MP_VH_DECL(mp_vb_c1)
MP_VH_DECL(mp_vb_c3)
MP_VH_DECL(mp_vb_c4)
MP_VH_DECL(mp_vd_c1)
MP_VH_DECL(mp_vd_c3)
MP_VH_DECL(mp_vd_c4)

int mp_vh_code(int cin, int cmid, int radius)
{
    int code = -1;
    if (cmid == 1 && (cin == 1 || cin == 3 || cin == 4)) code = cin;
    else if (cmid == cin && (cin == 3 || cin == 4)) code = 4 + cin;
    if (code < 0 || radius < 1 || radius > MP_VH_RBIG) return -1;
    // RGB channel-preserving radii 1..4 and 5..8 run on their own kernels
    // (code + 64, code + 128)
    if (code == 7 && radius <= 4) return code + 64;
    if (code == 7 && radius <= 8) return code + 128;
    if (radius <= MP_VH_RMAX) return code;
    // buckets: channel-keeping kernels only (1-channel source, RGB, RGBA)
    return (code == 1 || code == 7 || code == 8) ? code + 16 : -1;
}

int mp_vh_dot_code(int c, int radius)
{
    const int code = mp_vh_code(c, c, radius) & 63;   // the dot mode has one kernel for every radius
    return (code == 1 || code == 7 || code == 8) ? code + 32 : -1;
}

int mp_vh_bucket(int radius) { return radius <= MP_VH_RMAX ? radius : (radius <= 16 ? 16 : (radius <= 20 ? 20 : 24)); }

static int mp_vh_code_cin(int code) { code &= 15; return code > 4 ? code - 4 : code; }
static int mp_vh_code_cm(int code) { code &= 15; return code > 4 ? code - 4 : 1; }

static const void *mp_vh_fn(int code, bool single)
{
    switch (code) {
    case 1: return single ? (const void *)mp_vh_c1_single : (const void *)mp_vh_c1_batch;
    case 3: return single ? (const void *)mp_vh_c3_single : (const void *)mp_vh_c3_batch;
    case 4: return single ? (const void *)mp_vh_c4_single : (const void *)mp_vh_c4_batch;
    case 7: return single ? (const void *)mp_vc_c3_single : (const void *)mp_vc_c3_batch;
    case 7 + 64: return single ? (const void *)mp_vc_c3_lo_single : (const void *)mp_vc_c3_lo_batch;
    case 7 + 128: return single ? (const void *)mp_vc_c3_mid_single : (const void *)mp_vc_c3_mid_batch;
    case 8: return single ? (const void *)mp_vc_c4_single : (const void *)mp_vc_c4_batch;
    case 17: return single ? (const void *)mp_vb_c1_single : (const void *)mp_vb_c1_batch;
    case 23: return single ? (const void *)mp_vb_c3_single : (const void *)mp_vb_c3_batch;
    case 24: return single ? (const void *)mp_vb_c4_single : (const void *)mp_vb_c4_batch;
    case 33: return single ? (const void *)mp_vd_c1_single : (const void *)mp_vd_c1_batch;
    case 39: return single ? (const void *)mp_vd_c3_single : (const void *)mp_vd_c3_batch;
    case 40: return single ? (const void *)mp_vd_c4_single : (const void *)mp_vd_c4_batch;
    default: return nullptr;
    }
}

// Threads of a code's kernels: the radius buckets run 256 per CTA.
static int mp_vh_code_nt(int code) { return (code & 16) ? MP_VH_NT_BIG : MP_VH_NT; }

// Strip width limit; radii above MP_VH_RMAX run on the bucket kernels.
int mp_vh_strip(int radius, int cm)
{
    const int nt = radius > MP_VH_RMAX ? MP_VH_NT_BIG : MP_VH_NT;
    return 2 * nt - 2 * ((radius * cm + 3) & ~3);
}

// Strip width in columns for an image of width w pixels (w * cm columns):
// the fewest strips of at most mp_vh_strip(radius, cm) columns, evened out
// and rounded up to 8.
// Tuned cap on the strip width in columns (0: the kernel's limit).
static int mp_vh_strip_cap = 0;

void mp_vh_set_strip_cap(int cols) { mp_vh_strip_cap = cols; }

int mp_vh_fit_strip(int radius, int w, int cm)
{
    int maxw = mp_vh_strip(radius, cm);
    if (mp_vh_strip_cap >= 64 && mp_vh_strip_cap < maxw) maxw = mp_vh_strip_cap;
    const int wc = w * cm;
    const int n = (wc + maxw - 1) / maxw;
    const int sw = ((wc + n - 1) / n + 7) & ~7;
    return sw < 8 ? 8 : (sw > maxw ? maxw : sw);
}

size_t mp_vh_smem(int code)
{
    return (size_t)mp_vh::mp_vh_smem_floats(mp_vh_code_cin(code), mp_vh_code_cm(code), mp_vh_code_nt(code)) * 4 + 128;
}

MPStatus mp_vh_prepare(int code, int *ctas_per_sm)
{
    static std::mutex mtx;
    static std::vector<std::pair<const void *, int>> done;
    const void *fn = mp_vh_fn(code, false);
    if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return mp_cuda_status(e);
    {
        std::lock_guard<std::mutex> lk(mtx);
        bool have = false;
        for (auto &d : done)
            if (d.first == fn && d.second == dev) have = true;
        if (!have) {
            for (int single = 0; single < 2; ++single) {
                e = cudaFuncSetAttribute(mp_vh_fn(code, single != 0), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)mp_vh_smem(code));
                if (e != cudaSuccess) return mp_cuda_status(e);
            }
            done.push_back({fn, dev});
        }
    }
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, mp_vh_code_nt(code), mp_vh_smem(code));
    if (e != cudaSuccess) return mp_cuda_status(e);
    if (n < 1) return MP_ERROR_TOO_LARGE;
    *ctas_per_sm = n;
    return MILLIPYDE_SUCCESS;
}

MPStatus mp_vh_launch(int code, const MPJob *jobs_dev, const int *tile_job, int total, int grid, int *err,
                      int *counter, cudaStream_t s)
{
    if (total <= 0) return MILLIPYDE_SUCCESS;
    const void *fn = mp_vh_fn(code, false);
    if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
    if (grid > total) grid = total;
    if (grid < 1) grid = 1;
    void *args[] = {(void *)&jobs_dev, (void *)&tile_job, (void *)&total, (void *)&err, (void *)&counter};
    return mp_cuda_status(cudaLaunchKernel(fn, dim3(grid), dim3(mp_vh_code_nt(code)), args, mp_vh_smem(code), s));
}

MPStatus mp_vh_launch_single(int code, const MPJob &job, int grid, int *err, cudaStream_t s)
{
    if (job.ntiles <= 0) return MILLIPYDE_SUCCESS;
    const void *fn = mp_vh_fn(code, true);
    if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
    if (grid > job.ntiles) grid = job.ntiles;
    if (grid < 1) grid = 1;
    void *args[] = {(void *)&job, (void *)&err};
    return mp_cuda_status(cudaLaunchKernel(fn, dim3(grid), dim3(mp_vh_code_nt(code)), args, mp_vh_smem(code), s));
}
