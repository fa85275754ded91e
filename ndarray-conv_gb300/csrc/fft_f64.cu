// conv_fft and the FFT processor for double (one translation unit per element
// type, compiled in parallel).
#include "fft_entry.cuh"

namespace ndconv {
NDCONV_INST_FFT(double)
NDCONV_INST_PROC(double)
}  // namespace ndconv
