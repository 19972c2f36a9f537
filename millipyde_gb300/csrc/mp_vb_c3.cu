// mp_vb_c3.cu -- the streaming gaussian of mp_vh.cuh for radii above 12
// (buckets 16, 20, 24) on 3-channel images, channel count kept; one
// translation unit per channel count so the instances compile in parallel.
#include "mp_vh.cuh"

MP_VH_KERNELS_BIG(mp_vb_c3, 3, 3)
