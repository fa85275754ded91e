"""Python mirror of the ndarray-conv public types (src/lib.rs:67-159,
src/dilation/mod.rs:8-212).

Same names and argument meaning as the crate:

    ConvMode.Full / Same / Valid / Custom(padding, strides) / Explicit(padding, strides)
    PaddingMode.Zeros / Const(c) / Reflect / Replicate / Circular / Custom([...]) / Explicit([[..,..],...])
    BorderType.Zeros / Const(c) / Reflect / Replicate / Circular
    with_dilation(kernel, d).no_reverse()        (WithDilation, ReverseKernel)

and the crate's Error<N> variants as exceptions (DataShape, KernelShape,
MismatchShape), plus PaddingOutOfRange where the crate panics.
"""
from . import _abi


class ConvMode:
    """ConvMode<N> (src/lib.rs:81-105)."""

    def __init__(self, kind, padding=None, strides=None):
        self.kind = kind
        self.padding = padding
        self.strides = strides

    @staticmethod
    def Custom(padding, strides):
        return ConvMode(_abi.MODE_CUSTOM, list(padding), list(strides))

    @staticmethod
    def Explicit(padding, strides):
        return ConvMode(_abi.MODE_EXPLICIT, [list(p) for p in padding], list(strides))

    def __repr__(self):
        names = {0: "Full", 1: "Same", 2: "Valid", 3: "Custom", 4: "Explicit"}
        if self.kind in (_abi.MODE_CUSTOM, _abi.MODE_EXPLICIT):
            return f"ConvMode.{names[self.kind]}(padding={self.padding}, strides={self.strides})"
        return f"ConvMode.{names[self.kind]}"


ConvMode.Full = ConvMode(_abi.MODE_FULL)
ConvMode.Same = ConvMode(_abi.MODE_SAME)
ConvMode.Valid = ConvMode(_abi.MODE_VALID)


class BorderType:
    """BorderType<T> (src/lib.rs:131-143)."""

    def __init__(self, kind, value=0):
        self.kind = kind
        self.value = complex(value)

    @staticmethod
    def Const(c):
        return BorderType(_abi.BORDER_CONST, c)

    def __repr__(self):
        names = {0: "Zeros", 1: "Const", 2: "Reflect", 3: "Replicate", 4: "Circular"}
        if self.kind == _abi.BORDER_CONST:
            return f"BorderType.Const({self.value})"
        return f"BorderType.{names[self.kind]}"


BorderType.Zeros = BorderType(_abi.BORDER_ZEROS)
BorderType.Reflect = BorderType(_abi.BORDER_REFLECT)
BorderType.Replicate = BorderType(_abi.BORDER_REPLICATE)
BorderType.Circular = BorderType(_abi.BORDER_CIRCULAR)


class PaddingMode:
    """PaddingMode<N, T> (src/lib.rs:111-127)."""

    def __init__(self, kind, value=0, borders=None):
        self.kind = kind
        self.value = complex(value)
        self.borders = borders

    @staticmethod
    def Const(c):
        return PaddingMode(_abi.PAD_CONST, c)

    @staticmethod
    def Custom(borders):
        return PaddingMode(_abi.PAD_CUSTOM, borders=list(borders))

    @staticmethod
    def Explicit(borders):
        return PaddingMode(_abi.PAD_EXPLICIT, borders=[list(b) for b in borders])

    def __repr__(self):
        names = {0: "Zeros", 1: "Const", 2: "Reflect", 3: "Replicate", 4: "Circular",
                 5: "Custom", 6: "Explicit"}
        if self.kind == _abi.PAD_CONST:
            return f"PaddingMode.Const({self.value})"
        if self.kind in (_abi.PAD_CUSTOM, _abi.PAD_EXPLICIT):
            return f"PaddingMode.{names[self.kind]}({self.borders})"
        return f"PaddingMode.{names[self.kind]}"


PaddingMode.Zeros = PaddingMode(_abi.PAD_ZEROS)
PaddingMode.Reflect = PaddingMode(_abi.PAD_REFLECT)
PaddingMode.Replicate = PaddingMode(_abi.PAD_REPLICATE)
PaddingMode.Circular = PaddingMode(_abi.PAD_CIRCULAR)


class KernelWithDilation:
    """KernelWithDilation (src/dilation/mod.rs:8-12): kernel array, per-axis
    dilation, and the reverse flag (True = convolution, the default)."""

    def __init__(self, kernel, dilation=1, reverse=True):
        self.kernel = kernel
        nd = len(kernel.shape)
        if isinstance(dilation, int):
            dilation = [dilation] * nd
        self.dilation = list(dilation)
        self.reverse_flag = bool(reverse)

    def with_dilation(self, dilation):
        return KernelWithDilation(self.kernel, dilation, self.reverse_flag)

    def no_reverse(self):
        return KernelWithDilation(self.kernel, self.dilation, False)

    def reverse(self):
        return KernelWithDilation(self.kernel, self.dilation, True)


def into_kernel_with_dilation(k):
    """IntoKernelWithDilation (src/dilation/mod.rs:192-212): a bare array is
    dilation 1, reversed."""
    if isinstance(k, KernelWithDilation):
        return k
    return KernelWithDilation(k, 1, True)


def with_dilation(kernel, dilation):
    """WithDilation::with_dilation (src/dilation/mod.rs:103-126)."""
    return KernelWithDilation(kernel, dilation, True)


def no_reverse(kernel):
    """ReverseKernel::no_reverse (src/dilation/mod.rs:155-189)."""
    return into_kernel_with_dilation(kernel).no_reverse()


def reverse(kernel):
    """ReverseKernel::reverse (src/dilation/mod.rs:155-189)."""
    return into_kernel_with_dilation(kernel).reverse()


class ConvError(Exception):
    """Error<N> (src/lib.rs:148-159)."""

    def __init__(self, dims=None, detail=""):
        self.dims = tuple(dims) if dims is not None else None
        super().__init__(f"{type(self).__name__}({self.dims}) {detail}".strip())


class DataShape(ConvError):
    """Data shape shouldn't have ZERO (also the FFT path's zero-size kernel)."""


class KernelShape(ConvError):
    """Kernel shape shouldn't have ZERO (direct path)."""


class MismatchShape(ConvError):
    """ConvMode does not match the dilated kernel size."""


class PaddingOutOfRange(ConvError):
    """Where the crate panics (reflect padding index out of range)."""


class Unsupported(ConvError):
    pass


class CudaError(RuntimeError):
    pass


_NP_DTYPES = {"float32": _abi.F32, "float64": _abi.F64, "int32": _abi.I32,
              "complex64": _abi.C32, "complex128": _abi.C64, "int64": _abi.I64, "uint8": _abi.U8,
              "int8": _abi.I8, "int16": _abi.I16, "uint16": _abi.U16, "uint32": _abi.U32, "uint64": _abi.U64}


def dtype_code(dtype):
    """The ABI element type of a numpy / torch dtype.  Like the C ABI, element
    types outside f32, f64, c32, c64 and the 8- to 64-bit integers (e.g.
    float16, bool) raise Unsupported."""
    name = str(dtype).replace("torch.", "")
    if name not in _NP_DTYPES:
        raise Unsupported(None, f"element type {dtype} is not supported "
                                f"(f32, f64, c32, c64, i8, u8, i16, u16, i32, u32, i64, u64)")
    return _NP_DTYPES[name]


def build_problem(dtype, data_shape, kwd, conv_mode, padding_mode,
                  data_strides=None, kernel_strides=None):
    """Fill struct ndconv_problem from the mirrored types."""
    rank = len(data_shape)
    k = kwd.kernel
    if len(k.shape) != rank:
        raise ValueError("data and kernel rank differ")
    if rank > 3:
        raise Unsupported(None, "rank above 3 is not supported (ranks 1..3)")
    if rank < 1:
        raise ValueError("rank must be at least 1")
    p = _abi.Problem()
    p.dtype = dtype
    p.rank = rank
    for i in range(rank):
        p.data_shape[i] = int(data_shape[i])
        p.kernel_shape[i] = int(k.shape[i])
        p.dilation[i] = int(kwd.dilation[i])
    p.reverse = 1 if kwd.reverse_flag else 0
    p.conv_mode = conv_mode.kind
    if conv_mode.kind == _abi.MODE_CUSTOM:
        for i in range(rank):
            p.mode_padding[i][0] = p.mode_padding[i][1] = int(conv_mode.padding[i])
            p.mode_strides[i] = int(conv_mode.strides[i])
    elif conv_mode.kind == _abi.MODE_EXPLICIT:
        for i in range(rank):
            p.mode_padding[i][0] = int(conv_mode.padding[i][0])
            p.mode_padding[i][1] = int(conv_mode.padding[i][1])
            p.mode_strides[i] = int(conv_mode.strides[i])
    p.padding_mode = padding_mode.kind
    p.const_value[0] = padding_mode.value.real
    p.const_value[1] = padding_mode.value.imag
    if padding_mode.kind == _abi.PAD_CUSTOM:
        for i in range(rank):
            b = padding_mode.borders[i]
            for s in range(2):
                p.border_kind[i][s] = b.kind
                p.border_value[i][s][0] = b.value.real
                p.border_value[i][s][1] = b.value.imag
    elif padding_mode.kind == _abi.PAD_EXPLICIT:
        for i in range(rank):
            for s in range(2):
                b = padding_mode.borders[i][s]
                p.border_kind[i][s] = b.kind
                p.border_value[i][s][0] = b.value.real
                p.border_value[i][s][1] = b.value.imag
    if data_strides is not None:
        for i in range(rank):
            p.data_strides[i] = int(data_strides[i])
    if kernel_strides is not None:
        for i in range(rank):
            p.kernel_strides[i] = int(kernel_strides[i])
    return p


def raise_for_status(st, p, algo):
    """Map an ndconv_status to the mirrored Error<N> exception."""
    if st == _abi.OK:
        return
    rank = p.rank
    ds = tuple(p.data_shape[:rank])
    ks = tuple(p.kernel_shape[:rank])
    msg = _abi.last_error()
    if st == _abi.ERR_DATA_SHAPE:
        # the FFT path reports a zero-size kernel as DataShape(kernel dims)
        dims = ks if (algo == 1 and 0 in ks and 0 not in ds) else ds
        raise DataShape(dims, msg)
    if st == _abi.ERR_KERNEL_SHAPE:
        raise KernelShape(ks, msg)
    if st == _abi.ERR_MISMATCH_SHAPE:
        ke = tuple(ks[i] * p.dilation[i] - p.dilation[i] + 1 for i in range(rank))
        raise MismatchShape(ke, msg)
    if st == _abi.ERR_PAD_OUT_OF_RANGE:
        raise PaddingOutOfRange(ds, msg)
    if st == _abi.ERR_UNSUPPORTED:
        raise Unsupported(None, msg)
    if st == _abi.ERR_INVALID:
        raise ValueError(msg)
    raise CudaError(f"{_abi.STATUS_NAMES.get(st, st)}: {msg}")
