// mp_vc_c3_mid.cu -- channel-preserving streaming gaussian kernels for
// 3-channel interleaved images (see mp_vh.cuh, family CM = C), radii 5..8,
// 4 resident CTAs per SM.
#include "mp_vh.cuh"

MP_VH_KERNELS_MID(mp_vc_c3_mid, 3, 3)
