// mp_vc_c3_lo.cu -- channel-preserving streaming gaussian kernels for
// 3-channel interleaved images (see mp_vh.cuh, family CM = C), radii 1..4,
// 4 resident CTAs per SM.
#include "mp_vh.cuh"

MP_VH_KERNELS_LO(mp_vc_c3_lo, 3, 3)
