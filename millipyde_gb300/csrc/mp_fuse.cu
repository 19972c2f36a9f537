// mp_fuse.cu -- host side of the fused gaussian -> rotate kernel
// (mp_fuse.cuh; kernels in mp_fuse_c1.cu and mp_fuse_c3.cu).
#include <mutex>
#include <utility>
#include <vector>

#include "mp_internal.cuh"

__global__ void mp_fz_c1_batch(const MPJob *__restrict__, const int *__restrict__, int, const FzGeom, int *);
__global__ void mp_fz_c3_batch(const MPJob *__restrict__, const int *__restrict__, int, const FzGeom, int *);

static const void *mp_fz_fn(int cin)
{
    switch (cin) {
    case 1: return (const void *)mp_fz_c1_batch;
    case 3: return (const void *)mp_fz_c3_batch;
    default: return nullptr;
    }
}

bool mp_fz_supported(int cin, int radius) { return mp_fz_fn(cin) && radius >= 1 && radius <= MP_FZ_RMAX; }

// Layout (floats from the 128-byte aligned base): 32 floats of barriers,
// two chunk stages (the vertical pass's output V reuses them: 48 row pairs
// of 2 gp floats), then the plane G (96 + 2 rmax rows of gp floats; the
// horizontal pass's output B reuses it).
FzGeom mp_fz_geom(int box_max, int rmax, int cin, size_t *smem)
{
    FzGeom g;
    const int sw = box_max + 2 * rmax;                  // widest source region (pixels)
    g.gp = ((sw + 8 + 15) & ~15) + 4;                   // = 4 (mod 16): conflict-free row-pair loads
    const int nb = (3 + sw * cin + 127) / 128;          // boxes of 128 floats per chunk row
    g.stage = nb * 128 * MP_FZ_CR;
    int area = 2 * g.stage;
    if (area < 96 * g.gp) area = 96 * g.gp;
    g.offG = 32 + ((area + 31) & ~31);
    const int gh = 96 + 2 * rmax;
    if (smem) *smem = (size_t)(g.offG + gh * g.gp) * 4 + 128;
    return g;
}

MPStatus mp_fz_prepare(int cin, size_t smem, int *ctas_per_sm)
{
    static std::mutex mtx;
    static std::vector<std::pair<const void *, int>> done;
    const void *fn = mp_fz_fn(cin);
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
            int optin = 0;
            e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
            if (e != cudaSuccess) return mp_cuda_status(e);
            cudaFuncAttributes fa;
            e = cudaFuncGetAttributes(&fa, fn);
            if (e != cudaSuccess) return mp_cuda_status(e);
            e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
            if (e != cudaSuccess) return mp_cuda_status(e);
            done.push_back({fn, dev});
        }
    }
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, 256, smem);
    if (e != cudaSuccess) return mp_cuda_status(e);
    if (n < 1) return MP_ERROR_TOO_LARGE;
    *ctas_per_sm = n;
    return MILLIPYDE_SUCCESS;
}

MPStatus mp_fz_launch(int cin, const MPJob *jobs_dev, const int *tile_job, int total, const FzGeom &g, size_t smem,
                      int grid, int *err, cudaStream_t s)
{
    if (total <= 0) return MILLIPYDE_SUCCESS;
    const void *fn = mp_fz_fn(cin);
    if (!fn) return MP_ERROR_UNSUPPORTED_TYPE;
    if (grid > total) grid = total;
    if (grid < 1) grid = 1;
    FzGeom ga = g;
    void *args[] = {(void *)&jobs_dev, (void *)&tile_job, (void *)&total, (void *)&ga, (void *)&err};
    return mp_cuda_status(cudaLaunchKernel(fn, dim3(grid), dim3(256), args, smem, s));
}
