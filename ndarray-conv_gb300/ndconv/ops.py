"""conv / conv_fft / FFT processor over the C ABI (device tensors via torch).

Mirrors ConvExt::conv (src/conv/mod.rs:78-116), ConvFFTExt::{conv_fft,
conv_fft_with_processor, conv_fft_par} (src/conv_fft/mod.rs:81-183) and
get_fft_processor / Processor::{forward, backward}
(src/conv_fft/processor/mod.rs:71-143).  Inputs may be CUDA tensors (used
in place, any strides) or numpy arrays (copied to the GPU; the result comes
back as numpy).  Every call runs the CUDA library; there is no CPU path.
"""
import ctypes

import numpy as np
import torch

from . import _abi
from .api import build_problem, dtype_code, into_kernel_with_dilation, raise_for_status

_TORCH_OF = {_abi.F32: torch.float32, _abi.F64: torch.float64, _abi.I32: torch.int32,
             _abi.C32: torch.complex64, _abi.C64: torch.complex128}


# unsigned numpy types that travel to the device as their signed twin (the
# same bits; the ABI still gets the unsigned element type)
_SIGNED_TWIN = {np.dtype(np.uint16): np.int16, np.dtype(np.uint32): np.int32, np.dtype(np.uint64): np.int64}


def _to_device(a):
    if isinstance(a, torch.Tensor):
        if not a.is_cuda:
            return a.cuda(), True
        return a, False
    a = np.ascontiguousarray(a)
    if a.dtype in _SIGNED_TWIN:
        a = a.view(_SIGNED_TWIN[a.dtype])
    return torch.from_numpy(a).cuda(), True


def _np_dtype(a):
    """numpy dtype of a host array argument (None for tensors)."""
    return None if isinstance(a, torch.Tensor) else np.asarray(a).dtype


def _stream_ptr(stream):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _prepare(data, kernel, conv_mode, padding_mode):
    kwd = into_kernel_with_dilation(kernel)
    x, x_host = _to_device(data)
    k, _ = _to_device(kwd.kernel)
    if x.dtype != k.dtype:
        raise TypeError(f"data {x.dtype} and kernel {k.dtype} element types differ")
    nd = _np_dtype(data)
    dt = dtype_code(nd if nd is not None and nd in _SIGNED_TWIN else x.dtype)
    from .api import KernelWithDilation
    kwd = KernelWithDilation(k, kwd.dilation, kwd.reverse_flag)
    p = build_problem(dt, tuple(x.shape), kwd, conv_mode, padding_mode,
                      data_strides=x.stride(), kernel_strides=k.stride())
    return p, x, k, x_host


def _run(algo, data, kernel, conv_mode, padding_mode, processor=None, stream=None, variant=None):
    L = _abi.lib()
    p, x, k, x_host = _prepare(data, kernel, conv_mode, padding_mode)
    shape = (ctypes.c_int64 * 3)()
    raise_for_status(L.ndconv_output_shape(ctypes.byref(p), algo, shape), p, algo)
    y = torch.empty([shape[i] for i in range(p.rank)], dtype=x.dtype, device=x.device)
    sp = _stream_ptr(stream)
    if variant is not None:
        st = L.ndconv_conv_algo(ctypes.byref(p), variant, ctypes.c_void_p(x.data_ptr()),
                                ctypes.c_void_p(k.data_ptr()), ctypes.c_void_p(y.data_ptr()), sp)
    elif algo == 0:
        st = L.ndconv_conv(ctypes.byref(p), ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(k.data_ptr()),
                           ctypes.c_void_p(y.data_ptr()), sp)
    else:
        h = processor._handle if processor is not None else None
        st = L.ndconv_conv_fft(ctypes.byref(p), ctypes.c_void_p(x.data_ptr()),
                               ctypes.c_void_p(k.data_ptr()), ctypes.c_void_p(y.data_ptr()), h, sp)
    raise_for_status(st, p, algo)
    if x_host:
        out = y.cpu().numpy()
        nd = _np_dtype(data)
        return out.view(nd) if nd in _SIGNED_TWIN else out
    return y


def conv(data, kernel, conv_mode, padding_mode, stream=None):
    """ConvExt::conv: direct convolution (kernel may carry dilation/no_reverse)."""
    return _run(0, data, kernel, conv_mode, padding_mode, stream=stream)


def conv_fft(data, kernel, conv_mode, padding_mode, stream=None):
    """ConvFFTExt::conv_fft (f32, f64, complex64, complex128)."""
    return _run(1, data, kernel, conv_mode, padding_mode, stream=stream)


def conv_fft_with_processor(data, kernel, conv_mode, padding_mode, processor, stream=None):
    """ConvFFTExt::conv_fft_with_processor: reuses the processor's workspace."""
    return _run(1, data, kernel, conv_mode, padding_mode, processor=processor, stream=stream)


def conv_fft_par(data, kernel, conv_mode, padding_mode, stream=None):
    """ConvFFTExt::conv_fft_par: on the GPU the same kernels as conv_fft."""
    return _run(1, data, kernel, conv_mode, padding_mode, stream=stream)


def conv_algo(data, kernel, conv_mode, padding_mode, algo, stream=None):
    """One convolution by an explicit algorithm variant (ndconv_algo code,
    e.g. _abi.ALGO_FFT_RS); the autotuner times these."""
    base = 0 if algo in (_abi.ALGO_DIRECT, _abi.ALGO_DIRECT_BF16X3) else 1
    return _run(base, data, kernel, conv_mode, padding_mode, stream=stream, variant=int(algo))


class FftProcessor:
    """Processor<T, InElem> (src/conv_fft/processor/mod.rs:79-119)."""

    def __init__(self, dtype):
        self.dtype = dtype_code(dtype)
        h = ctypes.c_void_p()
        st = _abi.lib().ndconv_fft_processor_create(self.dtype, ctypes.byref(h))
        if st:
            raise RuntimeError(_abi.last_error())
        self._handle = h

    def close(self):
        if self._handle:
            _abi.lib().ndconv_fft_processor_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bake(self, data_like, kernel, conv_mode, padding_mode, stream=None):
        """Keep the kernel's spectrum for this geometry (the crate's sketched
        "baked" processor): later conv_fft_with_processor calls with the same
        geometry and the same kernel tensor skip the kernel transform.  The
        kernel must be a CUDA tensor; bake again after changing its contents."""
        kwd = into_kernel_with_dilation(kernel)
        if not (isinstance(kwd.kernel, torch.Tensor) and kwd.kernel.is_cuda):
            raise TypeError("bake needs the kernel as a CUDA tensor (its address is the key)")
        x = data_like if isinstance(data_like, torch.Tensor) else torch.empty(
            tuple(np.shape(data_like)), dtype=kwd.kernel.dtype)
        p = build_problem(dtype_code(kwd.kernel.dtype), tuple(x.shape), kwd, conv_mode, padding_mode,
                          kernel_strides=kwd.kernel.stride())
        st = _abi.lib().ndconv_fft_processor_bake(self._handle, ctypes.byref(p),
                                                  ctypes.c_void_p(kwd.kernel.data_ptr()), _stream_ptr(stream))
        raise_for_status(st, p, 1)
        self._baked = kwd.kernel  # keep the keyed tensor alive

    def _cdtype(self):
        return torch.complex64 if self.dtype in (_abi.F32, _abi.C32) else torch.complex128

    def forward(self, x, stream=None):
        """Spectrum in the reference's rotated axis layout."""
        xd, host = _to_device(x)
        xd = xd.contiguous()
        rank = xd.dim()
        shape = (ctypes.c_int64 * 3)(*list(xd.shape))
        osh = (ctypes.c_int64 * 3)()
        L = _abi.lib()
        st = L.ndconv_fft_forward(self._handle, rank, shape, None, None, osh, None)
        if st:
            raise RuntimeError(_abi.last_error())
        out = torch.empty([osh[i] for i in range(rank)], dtype=self._cdtype(), device=xd.device)
        st = L.ndconv_fft_forward(self._handle, rank, shape, ctypes.c_void_p(xd.data_ptr()),
                                  ctypes.c_void_p(out.data_ptr()), osh, _stream_ptr(stream))
        if st:
            raise RuntimeError(_abi.last_error())
        return out.cpu().numpy() if host else out

    def backward(self, spec, stream=None):
        sd, host = _to_device(spec)
        sd = sd.contiguous()
        rank = sd.dim()
        shape = (ctypes.c_int64 * 3)(*list(sd.shape))
        osh = (ctypes.c_int64 * 3)()
        L = _abi.lib()
        st = L.ndconv_fft_backward(self._handle, rank, shape, None, None, osh, None)
        if st:
            raise RuntimeError(_abi.last_error())
        odt = _TORCH_OF[self.dtype]
        out = torch.empty([osh[i] for i in range(rank)], dtype=odt, device=sd.device)
        st = L.ndconv_fft_backward(self._handle, rank, shape, ctypes.c_void_p(sd.data_ptr()),
                                   ctypes.c_void_p(out.data_ptr()), osh, _stream_ptr(stream))
        if st:
            raise RuntimeError(_abi.last_error())
        return out.cpu().numpy() if host else out


def get_fft_processor(dtype=torch.float32):
    """get_fft_processor::<T, InElem>() (src/lib.rs:75-77): real dtype -> real
    processor, complex dtype -> complex processor."""
    return FftProcessor(dtype)


def _ptr_array(tensors):
    return torch.tensor([t.data_ptr() for t in tensors], dtype=torch.int64, device=tensors[0].device)


def _run_batch(algo, datas, kernels, conv_mode, padding_mode, processor=None, stream=None):
    """One submission over instances that share shapes, dilation and modes."""
    L = _abi.lib()
    if len(datas) != len(kernels) or not datas:
        raise ValueError("need equally many data and kernel arrays (at least one)")
    kwd0 = into_kernel_with_dilation(kernels[0])
    xs = [_to_device(d)[0].contiguous() for d in datas]
    ks = [_to_device(into_kernel_with_dilation(k).kernel)[0].contiguous() for k in kernels]
    from .api import KernelWithDilation
    p = build_problem(dtype_code(xs[0].dtype), tuple(xs[0].shape),
                      KernelWithDilation(ks[0], kwd0.dilation, kwd0.reverse_flag), conv_mode, padding_mode)
    for x, k in zip(xs, ks):
        if tuple(x.shape) != tuple(xs[0].shape) or tuple(k.shape) != tuple(ks[0].shape) or x.dtype != xs[0].dtype:
            raise ValueError("batched instances must share shapes and element type")
    shape = (ctypes.c_int64 * 3)()
    base = 1 if algo == 1 else 0
    raise_for_status(L.ndconv_output_shape(ctypes.byref(p), base, shape), p, base)
    ys = [torch.empty([shape[i] for i in range(p.rank)], dtype=xs[0].dtype, device=xs[0].device)
          for _ in xs]
    px, pk, py = _ptr_array(xs), _ptr_array(ks), _ptr_array(ys)
    sp = _stream_ptr(stream)
    n = len(xs)
    if algo == 0:
        st = L.ndconv_conv_batch(ctypes.byref(p), n, ctypes.c_void_p(px.data_ptr()), ctypes.c_void_p(pk.data_ptr()),
                                 ctypes.c_void_p(py.data_ptr()), sp)
    elif algo == _abi.ALGO_DIRECT_BF16X3:
        st = L.ndconv_conv_bf16x3_batch(ctypes.byref(p), n, ctypes.c_void_p(px.data_ptr()),
                                        ctypes.c_void_p(pk.data_ptr()), ctypes.c_void_p(py.data_ptr()), sp)
    else:
        h = processor._handle if processor is not None else None
        st = L.ndconv_conv_fft_batch(ctypes.byref(p), n, ctypes.c_void_p(px.data_ptr()),
                                     ctypes.c_void_p(pk.data_ptr()), ctypes.c_void_p(py.data_ptr()), h, sp)
    raise_for_status(st, p, base)
    torch.cuda.current_stream().synchronize() if stream is None else stream.synchronize()
    return ys


def conv_batch(datas, kernels, conv_mode, padding_mode, stream=None):
    """conv over many instances with one geometry (kernels may carry the
    same dilation / no_reverse)."""
    return _run_batch(0, datas, kernels, conv_mode, padding_mode, stream=stream)


def conv_bf16x3_batch(datas, kernels, conv_mode, padding_mode, stream=None):
    """conv over many f32 instances with one geometry on the tensor cores
    (3xBF16 split products), one persistent launch for all of them."""
    return _run_batch(_abi.ALGO_DIRECT_BF16X3, datas, kernels, conv_mode, padding_mode, stream=stream)


def conv_fft_batch(datas, kernels, conv_mode, padding_mode, processor=None, stream=None):
    """conv_fft over many instances with one geometry, L2-sized waves."""
    return _run_batch(1, datas, kernels, conv_mode, padding_mode, processor=processor, stream=stream)


def conv_batch_host(xs, ks, ys, conv_mode, padding_mode, algo=1, processor=None, stream=None, sync=True):
    """conv (algo 0) / conv_fft (algo 1) over same-geometry instances held in
    HOST memory: xs, ks inputs and ys preallocated outputs, each a list of
    contiguous CPU torch tensors (pinned for full speed).  The library pipelines
    the copies with the convolution; `sync` waits for the stream."""
    L = _abi.lib()
    if not (len(xs) == len(ks) == len(ys)) or not xs:
        raise ValueError("need equally many data, kernel and output arrays (at least one)")
    kwd0 = into_kernel_with_dilation(ks[0])
    kt = [into_kernel_with_dilation(k).kernel for k in ks]
    from .api import KernelWithDilation
    p = build_problem(dtype_code(xs[0].dtype), tuple(xs[0].shape),
                      KernelWithDilation(kt[0], kwd0.dilation, kwd0.reverse_flag), conv_mode, padding_mode)
    n = len(xs)
    arr = ctypes.c_void_p * n
    px = arr(*[x.data_ptr() for x in xs])
    pk = arr(*[k.data_ptr() for k in kt])
    py = arr(*[y.data_ptr() for y in ys])
    h = processor._handle if processor is not None else None
    st = L.ndconv_conv_batch_host(ctypes.byref(p), algo, n, px, pk, py, h, _stream_ptr(stream))
    raise_for_status(st, p, algo)
    if sync:
        (stream or torch.cuda.current_stream()).synchronize()
    return ys
