// mp_vc_c3.cu -- channel-preserving streaming gaussian kernels for
// 3-channel interleaved images (see mp_vh.cuh, family CM = C), radii 9..12;
// radii 1..4 and 5..8 are separate kernels (mp_vc_c3_lo.cu, mp_vc_c3_mid.cu)
// with their own register allocation, compiled in parallel.
#include "mp_vh.cuh"

MP_VH_KERNELS_HI(mp_vc_c3, 3, 3)
