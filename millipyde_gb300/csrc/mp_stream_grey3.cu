// mp_stream_grey3.cu -- streaming gaussian kernels for 3-channel sources with an rgb2grey prologue (one translation unit
// per channel variant so the compiled-radius instances build in parallel).
#include "mp_stream.cuh"

MP_GS_KERNELS(mp_gs_grey3, 3, 1, 1)
