// mp_vc_c3.cu -- channel-preserving streaming gaussian kernels for
// 3-channel interleaved images (see mp_vh.cuh, family CM = C); one
// translation unit per channel count so the per-radius instances compile in
// parallel.
#include "mp_vh.cuh"

MP_VH_KERNELS(mp_vc_c3, 3, 3)
