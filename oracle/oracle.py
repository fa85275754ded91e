"""ctypes wrapper of the C oracle (oracle/ndconv_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference legs of bench.py as the oracle and the timed CPU
restatement of the reference.  The product never imports it.

Functions take a problem structure whose leading fields have the layout of
`orc_problem` (the library's `ndconv_problem` starts with the same fields)
and numpy arrays.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libndconv_oracle.so")

DT_F32, DT_F64, DT_I32, DT_C32, DT_C64 = 0, 1, 2, 3, 4
DT_I64, DT_U8, DT_I8, DT_I16, DT_U16, DT_U32, DT_U64 = 5, 6, 7, 8, 9, 10, 11
NP_OF = {DT_F32: np.float32, DT_F64: np.float64, DT_I32: np.int32,
         DT_C32: np.complex64, DT_C64: np.complex128, DT_I64: np.int64, DT_U8: np.uint8, DT_I8: np.int8,
         DT_I16: np.int16, DT_U16: np.uint16, DT_U32: np.uint32, DT_U64: np.uint64}

_lib = None


def build(force=False):
    """Compile the oracle with its Makefile (gcc, portable flags); make
    rebuilds it whenever a source, header or the Makefile is newer."""
    subprocess.run(["make", "-s"] + (["-B"] if force else []) + ["-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, i64p = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)
        L.orc_good_size.restype = ctypes.c_long
        L.orc_good_size.argtypes = [ctypes.c_long]
        L.orc_unfold.argtypes = [vp, i64p, i64p]
        L.orc_padding.argtypes = [vp, i64p, vp, ctypes.c_int, ctypes.c_int, vp]
        L.orc_taps.restype = ctypes.c_long
        L.orc_taps.argtypes = [vp, vp, ctypes.c_int, ctypes.POINTER(ctypes.c_long), vp, vp]
        L.orc_conv.argtypes = [vp, vp, vp, i64p, vp]
        L.orc_conv_fft.argtypes = [vp, vp, vp, i64p, vp, ctypes.c_int]
        L.orc_fft_forward.argtypes = [ctypes.c_int, ctypes.c_int, i64p, vp, vp, i64p, i64p]
        L.orc_fft_backward.argtypes = [ctypes.c_int, ctypes.c_int, i64p, vp, ctypes.c_int64, vp, i64p]
        L.orc_fft1d.argtypes = [ctypes.c_long, vp, vp, ctypes.c_int]
        L.orc_fft_buffers.argtypes = [vp, i64p, vp, vp, vp, vp]
        _lib = L
    return _lib


def _i64(vals, n=3):
    a = (ctypes.c_int64 * n)()
    for i, v in enumerate(vals):
        a[i] = int(v)
    return a


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _as(arr, dt):
    return np.ascontiguousarray(np.asarray(arr), dtype=NP_OF[dt])


def good_size(n):
    """good_size_cc (src/conv_fft/good_size.rs:6-31)."""
    return int(lib().orc_good_size(int(n)))


def unfold(p):
    """ConvMode::unfold -> (padding [[p0,p1]..], strides)."""
    pad = (ctypes.c_int64 * 6)()
    st = (ctypes.c_int64 * 3)()
    lib().orc_unfold(ctypes.byref(p), pad, st)
    r = p.rank
    return [[pad[2 * i], pad[2 * i + 1]] for i in range(r)], [st[i] for i in range(r)]


def padding(p, x, fft_style=False, pad=None):
    """PaddingExt::padding (fft_style False) / padding_in into a zeroed buffer
    (True).  x: real or complex numpy array.  Returns (status, padded)."""
    x = np.asarray(x)
    cplx = np.iscomplexobj(x)
    nc = 2 if cplx else 1
    if pad is None:
        pad, _ = unfold(p)
    r = p.rank
    xd = np.ascontiguousarray(x, dtype=np.complex128 if cplx else np.float64)
    L = [x.shape[i] + pad[i][0] + pad[i][1] for i in range(r)]
    out = np.zeros(L, dtype=xd.dtype)
    padc = _i64([v for pr in pad for v in pr], 6)
    st = lib().orc_padding(ctypes.byref(p), padc, _ptr(xd), nc, 1 if fft_style else 0, _ptr(out))
    return st, out


def taps(p, k, pds_strides):
    """gen_offset_list -> list of (offset, value)."""
    k = np.asarray(k)
    cplx = np.iscomplexobj(k)
    kd = np.ascontiguousarray(k, dtype=np.complex128 if cplx else np.float64)
    n = kd.size
    offs = (ctypes.c_long * (n + 1))()
    vals = np.zeros(n + 1, dtype=kd.dtype)
    strides = (ctypes.c_long * 3)(*[int(s) for s in pds_strides])
    cnt = lib().orc_taps(ctypes.byref(p), _ptr(kd), 2 if cplx else 1, strides, offs, _ptr(vals))
    return [(offs[i], vals[i]) for i in range(cnt)]


def conv(p, x, k):
    """ConvExt::conv in the problem's dtype.  Returns (status, y)."""
    dt = p.dtype
    xa, ka = _as(x, dt), _as(k, dt)
    ys = (ctypes.c_int64 * 3)()
    st = lib().orc_conv(ctypes.byref(p), _ptr(xa), _ptr(ka), ys, None)
    if st:
        return st, None
    y = np.zeros([ys[i] for i in range(p.rank)], dtype=NP_OF[dt])
    st = lib().orc_conv(ctypes.byref(p), _ptr(xa), _ptr(ka), ys, _ptr(y))
    return st, y


def conv_fft(p, x, k, nthreads=1):
    """conv_fft (nthreads 1) / conv_fft_par (nthreads > 1). (status, y)."""
    dt = p.dtype
    xa, ka = _as(x, dt), _as(k, dt)
    ys = (ctypes.c_int64 * 3)()
    st = lib().orc_conv_fft(ctypes.byref(p), _ptr(xa), _ptr(ka), ys, None, 1)
    if st:
        return st, None
    y = np.zeros([ys[i] for i in range(p.rank)], dtype=NP_OF[dt])
    st = lib().orc_conv_fft(ctypes.byref(p), _ptr(xa), _ptr(ka), ys, _ptr(y), int(nthreads))
    return st, y


def fft_forward(dt, x):
    """Processor::forward -> (spectrum in the rotated layout, origin_len)."""
    xa = _as(x, dt)
    r = xa.ndim
    s = _i64(xa.shape)
    cdt = np.complex64 if dt in (DT_F32, DT_C32) else np.complex128
    shp = list(xa.shape)
    if dt in (DT_F32, DT_F64):
        shp[-1] = shp[-1] // 2 + 1
    out = np.zeros(int(np.prod(shp)), dtype=cdt)
    osh = (ctypes.c_int64 * 3)()
    ol = ctypes.c_int64()
    lib().orc_fft_forward(dt, r, s, _ptr(xa), _ptr(out), osh, ctypes.byref(ol))
    return out.reshape([osh[i] for i in range(r)]), ol.value


def fft_backward(dt, spec, origin_len):
    """Processor::backward of a rotated-layout spectrum."""
    cdt = np.complex64 if dt in (DT_F32, DT_C32) else np.complex128
    sa = np.ascontiguousarray(spec, dtype=cdt)
    r = sa.ndim
    if dt in (DT_F32, DT_F64):
        # the real output count is (size / h) * origin_len <= 2 * size
        out = np.zeros(2 * sa.size + 8, dtype=np.float32 if dt == DT_F32 else np.float64)
    else:
        out = np.zeros(sa.size, dtype=cdt)
    osh = (ctypes.c_int64 * 3)()
    lib().orc_fft_backward(dt, r, _i64(sa.shape), _ptr(sa), int(origin_len), _ptr(out), osh)
    shp = [osh[i] for i in range(r)]
    return out[:int(np.prod(shp))].reshape(shp)


def fft1d(x, inverse=False):
    """The oracle's own unnormalised 1-D complex FFT (f64)."""
    xa = np.ascontiguousarray(x, dtype=np.complex128)
    out = np.zeros_like(xa)
    lib().orc_fft1d(xa.size, _ptr(xa), _ptr(out), 1 if inverse else -1)
    return out


def fft_buffers(p, fft_size, x, k):
    """padding::data / padding::kernel buffers (real)."""
    xa = np.ascontiguousarray(x, dtype=np.float64)
    ka = np.ascontiguousarray(k, dtype=np.float64)
    d = np.zeros(fft_size, dtype=np.float64)
    kb = np.zeros(fft_size, dtype=np.float64)
    st = lib().orc_fft_buffers(ctypes.byref(p), _i64(fft_size), _ptr(xa), _ptr(ka), _ptr(d), _ptr(kb))
    return st, d, kb
