"""ndconv: GB300 (sm_103a) drop-in for the ndarray-conv convolution hot path.

Python mirror of the crate's API over the C ABI in include/ndconv.h.
"""
from .api import (BorderType, ConvError, ConvMode, DataShape, KernelShape,  # noqa: F401
                  KernelWithDilation, MismatchShape, PaddingMode, PaddingOutOfRange,
                  Unsupported, build_problem, no_reverse, reverse, with_dilation)
from .ops import (FftProcessor, conv, conv_algo, conv_batch, conv_batch_host, conv_bf16x3_batch, conv_fft, conv_fft_batch, conv_fft_par,  # noqa: F401,E402
                  conv_fft_with_processor, get_fft_processor)
