"""Shared helpers for the parity tests (problem construction, error norms)."""
import numpy as np

from ndconv import BorderType, ConvMode, PaddingMode, build_problem, with_dilation  # noqa: F401
from ndconv import _abi
from ndconv.api import KernelWithDilation, into_kernel_with_dilation


def mode_from_json(m):
    if m[0] == "Full":
        return ConvMode.Full
    if m[0] == "Same":
        return ConvMode.Same
    if m[0] == "Valid":
        return ConvMode.Valid
    if m[0] == "Custom":
        return ConvMode.Custom(m[1], m[2])
    return ConvMode.Explicit(m[1], m[2])


def problem(dtype, x, kernel, conv_mode, padding_mode, data_strides=None):
    """ndconv_problem for data array x and kernel (array or KernelWithDilation)."""
    kwd = into_kernel_with_dilation(kernel)
    return build_problem(dtype, np.shape(x), kwd, conv_mode, padding_mode,
                         data_strides=data_strides)


def kernel_array(kernel):
    return into_kernel_with_dilation(kernel).kernel


def normwise_err(y, y64):
    """||y - y64||_2 / ||y64||_2 in float64."""
    y = np.asarray(y).astype(np.complex128 if np.iscomplexobj(y) else np.float64)
    y64 = np.asarray(y64).astype(np.complex128 if np.iscomplexobj(y64) else np.float64)
    den = np.linalg.norm(y64.ravel())
    num = np.linalg.norm((y - y64).ravel())
    return num / den if den > 0 else num


F32, F64, I32, C32, C64 = _abi.F32, _abi.F64, _abi.I32, _abi.C32, _abi.C64
__all__ = ["problem", "normwise_err", "mode_from_json", "KernelWithDilation", "with_dilation",
           "BorderType", "ConvMode", "PaddingMode", "F32", "F64", "I32", "C32", "C64", "kernel_array"]
