// mp_vd_c1.cu -- the d sigma dot mode of the streaming gaussian of
// mp_vh.cuh on 1-channel images (radii 1..12); one translation unit per
// channel count so the instances compile in parallel.
#include "mp_vh.cuh"

MP_VH_KERNELS_DOT(mp_vd_c1, 1, 1)
