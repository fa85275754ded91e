"""ctypes view of the C ABI declared in include/ndconv.h.

Loads the in-tree ``libndconv.so`` built for sm_103a.  There is no CPU
fallback: if the shared library is missing, every entry point raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "_build", "libndconv.so")

# ndconv_dtype
F32, F64, I32, C32, C64 = 0, 1, 2, 3, 4
I64, U8, I8, I16, U16, U32, U64 = 5, 6, 7, 8, 9, 10, 11  # integer types beyond i32: ndconv_conv only
# ndconv_status
# ndconv_algo: algorithm variants (autotuner candidates)
ALGO_DIRECT, ALGO_FFT, ALGO_DIRECT_BF16X3 = 0, 1, 2
ALGO_FFT_ND, ALGO_FFT_RS, ALGO_FFT_ND_POW2, ALGO_FFT_RS_POW2 = 3, 4, 5, 6
ALGO_NAMES = {0: "direct", 1: "fft", 2: "direct_bf16x3", 3: "fft_nd", 4: "fft_rs", 5: "fft_nd_pow2",
              6: "fft_rs_pow2"}

OK = 0
ERR_DATA_SHAPE = 1
ERR_KERNEL_SHAPE = 2
ERR_MISMATCH_SHAPE = 3
ERR_PAD_OUT_OF_RANGE = 4
ERR_UNSUPPORTED = 5
ERR_INVALID = 6
ERR_CUDA = 7
ERR_TIMEOUT = 8
ERR_NO_MEMORY = 9

# ndconv_tune_knob
TUNE_SW_TY, TUNE_MAC_ROWS, TUNE_ROW_THREADS, TUNE_BF16X3_BN, TUNE_SW_RY = 0, 1, 2, 3, 4
STATUS_NAMES = {
    0: "OK", 1: "DATA_SHAPE", 2: "KERNEL_SHAPE", 3: "MISMATCH_SHAPE",
    4: "PAD_OUT_OF_RANGE", 5: "UNSUPPORTED", 6: "INVALID", 7: "CUDA",
    8: "TIMEOUT", 9: "NO_MEMORY",
}
# ndconv_conv_mode
MODE_FULL, MODE_SAME, MODE_VALID, MODE_CUSTOM, MODE_EXPLICIT = 0, 1, 2, 3, 4
# ndconv_border
BORDER_ZEROS, BORDER_CONST, BORDER_REFLECT, BORDER_REPLICATE, BORDER_CIRCULAR = 0, 1, 2, 3, 4
# ndconv_padding_mode
PAD_ZEROS, PAD_CONST, PAD_REFLECT, PAD_REPLICATE, PAD_CIRCULAR, PAD_CUSTOM, PAD_EXPLICIT = range(7)

I64x3 = ctypes.c_int64 * 3


class Problem(ctypes.Structure):
    """struct ndconv_problem (include/ndconv.h)."""

    _fields_ = [
        ("dtype", ctypes.c_int32),
        ("rank", ctypes.c_int32),
        ("data_shape", ctypes.c_int64 * 3),
        ("kernel_shape", ctypes.c_int64 * 3),
        ("dilation", ctypes.c_int64 * 3),
        ("reverse", ctypes.c_int32),
        ("conv_mode", ctypes.c_int32),
        ("mode_padding", (ctypes.c_int64 * 2) * 3),
        ("mode_strides", ctypes.c_int64 * 3),
        ("padding_mode", ctypes.c_int32),
        ("border_kind", (ctypes.c_int32 * 2) * 3),
        ("border_value", ((ctypes.c_double * 2) * 2) * 3),
        ("const_value", ctypes.c_double * 2),
        ("data_strides", ctypes.c_int64 * 3),
        ("kernel_strides", ctypes.c_int64 * 3),
    ]


_lib = None


def lib():
    """The loaded libndconv.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"ndconv CUDA library not found at {LIB_PATH}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(LIB_PATH)
    vp, i32, i64p = ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)
    fp = ctypes.POINTER(ctypes.c_float)
    pp = ctypes.POINTER(Problem)
    sig = {
        "ndconv_output_shape": (ctypes.c_int, [pp, i32, i64p]),
        "ndconv_conv": (ctypes.c_int, [pp, vp, vp, vp, vp]),
        "ndconv_padded_host": (ctypes.c_int, [pp, vp, i32, vp]),
        "ndconv_conv_fft": (ctypes.c_int, [pp, vp, vp, vp, vp, vp]),
        "ndconv_conv_fft_noalloc": (ctypes.c_int, [pp, vp, vp, vp, vp]),
        "ndconv_conv_algo": (ctypes.c_int, [pp, i32, vp, vp, vp, vp]),
        "ndconv_conv_batch_host": (ctypes.c_int, [pp, i32, ctypes.c_int64, vp, vp, vp, vp, vp]),
        "ndconv_fft_processor_bake": (ctypes.c_int, [vp, pp, vp, vp]),
        "ndconv_conv_batch": (ctypes.c_int, [pp, ctypes.c_int64, vp, vp, vp, vp]),
        "ndconv_conv_fft_batch": (ctypes.c_int, [pp, ctypes.c_int64, vp, vp, vp, vp, vp]),
        "ndconv_fft_processor_create": (ctypes.c_int, [i32, ctypes.POINTER(vp)]),
        "ndconv_fft_processor_destroy": (ctypes.c_int, [vp]),
        "ndconv_fft_forward": (ctypes.c_int, [vp, i32, i64p, vp, vp, i64p, vp]),
        "ndconv_fft_backward": (ctypes.c_int, [vp, i32, i64p, vp, vp, i64p, vp]),
        "ndconv_last_error": (ctypes.c_char_p, []),
        "ndconv_version": (ctypes.c_char_p, []),
        "ndconv_kernel_launches": (ctypes.c_uint64, []),
        "ndconv_batch_create": (ctypes.c_int, [pp, ctypes.c_int64, vp, vp, vp, vp, ctypes.POINTER(vp)]),
        "ndconv_batch_run": (ctypes.c_int, [vp, i32, vp]),
        "ndconv_batch_run_plain": (ctypes.c_int, [vp, vp]),
        "ndconv_batch_status": (ctypes.c_int, [vp, vp]),
        "ndconv_batch_set_wait_limit": (ctypes.c_int, [vp, ctypes.c_int64]),
        "ndconv_batch_stall_one_wait": (ctypes.c_int, [vp, i32]),
        "ndconv_bf16x3_status": (ctypes.c_int, [vp]),
        "ndconv_conv_bf16x3_batch": (ctypes.c_int, [pp, ctypes.c_int64, vp, vp, vp, vp]),
        "ndconv_bf16x3_plan": (ctypes.c_int, [pp, i64p]),
        "ndconv_set_tuning": (ctypes.c_int, [i32, i32]),
        "ndconv_get_tuning": (ctypes.c_int32, [i32]),
        "ndconv_batch_info": (ctypes.c_int, [vp, i64p]),
        "ndconv_batch_destroy": (ctypes.c_int, [vp]),
        "ndconv_plan_info": (ctypes.c_int, [pp, ctypes.POINTER(ctypes.c_double)]),
        "ndconv_mlp_create": (ctypes.c_int, [i32, i32, i32, ctypes.c_uint64, ctypes.POINTER(vp)]),
        "ndconv_mlp_destroy": (ctypes.c_int, [vp]),
        "ndconv_mlp_param_count": (ctypes.c_int64, [vp]),
        "ndconv_mlp_params": (ctypes.c_int, [vp, fp, ctypes.c_int64, i32]),
        "ndconv_mlp_forward": (ctypes.c_int, [vp, fp, ctypes.c_int64, fp, vp]),
        "ndconv_mlp_gradient": (ctypes.c_int, [vp, fp, fp, fp, ctypes.c_int64, fp, fp, vp]),
        "ndconv_mlp_train": (ctypes.c_int, [vp, fp, fp, fp, ctypes.c_int64, i32, i32, ctypes.c_float,
                                            ctypes.c_uint64, fp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def last_error():
    return lib().ndconv_last_error().decode("utf-8", "replace")
