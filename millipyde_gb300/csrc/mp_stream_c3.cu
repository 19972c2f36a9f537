// mp_stream_c3.cu -- streaming gaussian kernels for 3-channel images (one translation unit
// per channel variant so the compiled-radius instances build in parallel).
#include "mp_stream.cuh"

MP_GS_KERNELS(mp_gs_c3, 3, 3, 1)
