// mp_fuse_c3.cu -- fused gaussian -> rotate kernel for 3-channel sources
// whose prologue ends in rgb2grey (see mp_fuse.cuh); one translation unit
// per source channel count so the per-radius instances compile in parallel.
#include "mp_fuse.cuh"

MP_FZ_KERNEL(mp_fz_c3_batch, 3)
