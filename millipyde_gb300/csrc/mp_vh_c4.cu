// mp_vh_c4.cu -- single-channel streaming gaussian kernels for 4-channel
// sources (see mp_vh.cuh); one translation unit per source channel count
// so the per-radius instances compile in parallel.
#include "mp_vh.cuh"

MP_VH_KERNELS(mp_vh_c4, 4, 1)
