// conv_fft and the FFT processor for float (one translation unit per element
// type, compiled in parallel).
#include "fft_entry.cuh"

namespace ndconv {
NDCONV_INST_FFT(float)
NDCONV_INST_PROC(float)
}  // namespace ndconv
