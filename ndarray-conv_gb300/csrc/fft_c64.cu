// conv_fft and the FFT processor for c64 (one translation unit per element
// type, compiled in parallel).
#include "fft_entry.cuh"

namespace ndconv {
NDCONV_INST_FFT(c64)
NDCONV_INST_PROC(c64)
}  // namespace ndconv
