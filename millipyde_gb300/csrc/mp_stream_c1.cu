// mp_stream_c1.cu -- streaming gaussian kernels for 1-channel images (one translation unit
// per channel variant so the compiled-radius instances build in parallel).
#include "mp_stream.cuh"

MP_GS_KERNELS(mp_gs_c1, 1, 1, 1)
