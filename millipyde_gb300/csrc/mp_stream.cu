// mp_stream.cu -- host side of the streaming gaussian, and the kernels of
// the 4-channel variants (loop passes only; the compiled-radius kernels of
// the other variants are in mp_stream_c1.cu, mp_stream_c3.cu and
// mp_stream_grey3.cu, built from mp_stream.cuh).
#include <mutex>
#include <utility>
#include <vector>

#include "mp_stream.cuh"

MP_GS_KERNELS(mp_gs_c4, 4, 4, 0)
MP_GS_KERNELS(mp_gs_grey4, 4, 1, 0)

#define MP_GS_DECL(NAME)                                                                            \
    __global__ void NAME##_batch(const MPJob *__restrict__, const int *__restrict__, int, const GsGeom, int *); \
    __global__ void NAME##_single(const MPJob, const GsGeom, int *);
MP_GS_DECL(mp_gs_c1)
MP_GS_DECL(mp_gs_c3)
MP_GS_DECL(mp_gs_grey3)

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static const void *mp_gs_fn(int variant, bool single)
{
    // variant numbering follows mp_variant: 0 c1, 1 c3, 2 c4, 3 grey3, 4 grey4
    static const void *batch[5] = {(const void *)mp_gs_c1_batch, (const void *)mp_gs_c3_batch,
                                   (const void *)mp_gs_c4_batch, (const void *)mp_gs_grey3_batch,
                                   (const void *)mp_gs_grey4_batch};
    static const void *one[5] = {(const void *)mp_gs_c1_single, (const void *)mp_gs_c3_single,
                                 (const void *)mp_gs_c4_single, (const void *)mp_gs_grey3_single,
                                 (const void *)mp_gs_grey4_single};
    if (variant < 0 || variant > 4) return nullptr;
    return single ? one[variant] : batch[variant];
}

static int mp_gs_threads(int variant)
{
    static const int cmid[5] = {1, 3, 4, 1, 1};
    return (variant >= 0 && variant < 5) ? mp_gs_nt(cmid[variant]) : 0;
}

// Raises the dynamic shared-memory limit of both kernels of a variant to the
// device's opt-in maximum (once per kernel and device) and reports how many
// CTAs of `smem` bytes fit on one SM.
MPStatus mp_gs_prepare(int variant, size_t smem, int *ctas_per_sm)
{
    static std::mutex mtx;
    static std::vector<std::pair<const void *, int>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return mp_cuda_status(e);
    for (int single = 0; single < 2; ++single) {
        const void *fn = mp_gs_fn(variant, single != 0);
        if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
        std::lock_guard<std::mutex> lk(mtx);
        bool have = false;
        for (auto &d : done)
            if (d.first == fn && d.second == dev) have = true;
        if (have) continue;
        int optin = 0;
        e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return mp_cuda_status(e);
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        if (e != cudaSuccess) return mp_cuda_status(e);
        done.push_back({fn, dev});
    }
    if (ctas_per_sm) {
        int n = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, mp_gs_fn(variant, false), mp_gs_threads(variant),
                                                          smem);
        if (e != cudaSuccess) return mp_cuda_status(e);
        if (n < 1) return MP_ERROR_TOO_LARGE;
        *ctas_per_sm = n;
    }
    return MILLIPYDE_SUCCESS;
}

MPStatus mp_gs_launch(int variant, const MPJob *jobs_dev, const int *tile_job, int total, const GsGeom &g,
                      int grid, int *err, cudaStream_t s)
{
    if (total <= 0) return MILLIPYDE_SUCCESS;
    const void *fn = mp_gs_fn(variant, false);
    if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
    if (grid > total) grid = total;
    if (grid < 1) grid = 1;
    GsGeom gg = g;
    void *args[] = {(void *)&jobs_dev, (void *)&tile_job, (void *)&total, (void *)&gg, (void *)&err};
    return mp_cuda_status(
        cudaLaunchKernel(fn, dim3(grid), dim3(mp_gs_threads(variant)), args, (size_t)g.total + 128, s));
}

MPStatus mp_gs_launch_single(int variant, const MPJob &job, const GsGeom &g, int grid, int *err, cudaStream_t s)
{
    if (job.ntiles <= 0) return MILLIPYDE_SUCCESS;
    const void *fn = mp_gs_fn(variant, true);
    if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
    if (grid > job.ntiles) grid = job.ntiles;
    if (grid < 1) grid = 1;
    GsGeom gg = g;
    void *args[] = {(void *)&job, (void *)&gg, (void *)&err};
    return mp_cuda_status(
        cudaLaunchKernel(fn, dim3(grid), dim3(mp_gs_threads(variant)), args, (size_t)g.total + 128, s));
}
