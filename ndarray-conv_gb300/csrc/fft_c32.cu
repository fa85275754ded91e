// conv_fft and the FFT processor for c32 (one translation unit per element
// type, compiled in parallel).
#include "fft_entry.cuh"

namespace ndconv {
NDCONV_INST_FFT(c32)
NDCONV_INST_PROC(c32)
}  // namespace ndconv
