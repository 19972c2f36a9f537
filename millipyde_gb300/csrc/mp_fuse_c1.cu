// mp_fuse_c1.cu -- fused gaussian -> rotate kernel for 1-channel sources
// (see mp_fuse.cuh); one translation unit per source channel count so the
// per-radius instances compile in parallel.
#include "mp_fuse.cuh"

MP_FZ_KERNEL(mp_fz_c1_batch, 1)
