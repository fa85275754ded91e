"""ndconv_conv_fft_noalloc: FFT convolution for callers that cannot allocate.

Real-time hosts that forbid device allocation after start-up, and plugins
whose host application owns every allocation, cannot let the library call
cudaMalloc.  This entry point uses a fixed 16 MiB device array inside the
library instead.  Its results must match ndconv_conv_fft (the allocating
entry point) within the tests' f32 tolerance, on two calls in a row, after
another call of a different geometry and element type has left NaN across
the shared array; one case is also checked against the f64 oracle.  The
calls must allocate nothing (device free memory and the default memory
pool's high-water mark unchanged), oversize problems must be rejected, and
problems no FFT form can take get NDCONV_ERR_UNSUPPORTED where
ndconv_conv_fft would fall back to the (allocating) direct kernels.
Collected last so a failure here leaves every other test already run;
passes alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

from helpers import F64, BorderType, ConvMode, PaddingMode, normwise_err, problem, with_dilation
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL32 = 1e-5


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build()
    from ndconv import _abi
    return _abi.lib()


def _call(lib, fn, p, x, k, y, *extra):
    import torch
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = [ctypes.byref(p), ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(k.data_ptr()),
            ctypes.c_void_p(y.data_ptr())] + list(extra) + [sp]
    return getattr(lib, fn)(*args)


class _PoolWatch:
    """High-water mark of the device's default memory pool (stream-ordered
    allocations), through the CUDA runtime the process already loaded."""

    USED_MEM_HIGH = 8  # cudaMemPoolAttrUsedMemHigh

    def __init__(self):
        self.rt, self.pool = None, ctypes.c_void_p()
        for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
            try:
                rt = ctypes.CDLL(name)
            except OSError:
                continue
            import torch
            if rt.cudaDeviceGetDefaultMemPool(ctypes.byref(self.pool), torch.cuda.current_device()) == 0:
                self.rt = rt
                break

    def reset(self):
        if self.rt:
            v = ctypes.c_uint64(0)
            assert self.rt.cudaMemPoolSetAttribute(self.pool, self.USED_MEM_HIGH, ctypes.byref(v)) == 0

    def high(self):
        if not self.rt:
            return 0
        v = ctypes.c_uint64(0)
        assert self.rt.cudaMemPoolGetAttribute(self.pool, self.USED_MEM_HIGH, ctypes.byref(v)) == 0
        return v.value


def _scribble(lib):
    """A noalloc call of another geometry and element type whose spectra are
    NaN, spread over most of the shared array."""
    import torch
    from ndconv import _abi, build_problem
    xs, ks = (420, 3000), (5, 7)
    x = torch.full(xs, float("nan"), device="cuda", dtype=torch.float64)
    k = torch.full(ks, 1e300, device="cuda", dtype=torch.float64)
    y = torch.empty(xs, device="cuda", dtype=torch.float64)
    p = build_problem(_abi.F64, xs, with_dilation(k, 1), ConvMode.Same, PaddingMode.Replicate)
    st = _call(lib, "ndconv_conv_fft_noalloc", p, x, k, y)
    if st == _abi.ERR_NO_MEMORY:  # keep under the array's size
        xs = (200, 3000)
        x, y = x[:200].contiguous(), y[:200].contiguous()
        p = build_problem(_abi.F64, xs, with_dilation(k, 1), ConvMode.Same, PaddingMode.Replicate)
        st = _call(lib, "ndconv_conv_fft_noalloc", p, x, k, y)
    assert st == 0, _abi.last_error()
    torch.cuda.synchronize()
    assert torch.isnan(y).all()


CASES = [
    ("2d_f32", (200, 5000), (11, 31), 2, ConvMode.Same,
     PaddingMode.Custom([BorderType.Reflect, BorderType.Circular]), "float32"),
    ("3d_c32", (10, 40, 50), (3, 5, 7), 1, ConvMode.Full, PaddingMode.Replicate, "complex64"),
    ("1d_f64", (4000,), (31,), 3, ConvMode.Custom([20], [2]), PaddingMode.Reflect, "float64"),
]


@pytest.mark.parametrize("name,xs,ks,dil,mode,pm,dt", CASES)
def test_noalloc_matches_conv_fft_on_two_calls(lib, name, xs, ks, dil, mode, pm, dt):
    import torch
    from ndconv import _abi, build_problem
    g = torch.Generator(device="cuda").manual_seed(len(name))
    tdt = getattr(torch, dt)
    if tdt.is_complex:
        x = torch.randn(xs, generator=g, device="cuda", dtype=tdt)
        k = torch.randn(ks, generator=g, device="cuda", dtype=tdt)
    else:
        x = torch.rand(xs, generator=g, device="cuda", dtype=tdt)
        k = torch.rand(ks, generator=g, device="cuda", dtype=tdt)
    from ndconv.api import dtype_code
    p = build_problem(dtype_code(tdt), xs, with_dilation(k, dil), mode, pm)
    osh = (ctypes.c_int64 * 3)()
    assert lib.ndconv_output_shape(ctypes.byref(p), 1, osh) == 0
    shape = [osh[i] for i in range(len(xs))]
    y_ref = torch.empty(shape, device="cuda", dtype=tdt)
    assert _call(lib, "ndconv_conv_fft", p, x, k, y_ref, None) == 0, _abi.last_error()
    outs = [torch.full(shape, float("nan"), device="cuda", dtype=tdt) for _ in range(2)]
    _scribble(lib)
    # nothing is allocated by the calls: device free memory and the default
    # pool's high-water mark stay as they were
    pool = _PoolWatch()
    torch.cuda.synchronize()
    pool.reset()
    free0 = torch.cuda.mem_get_info()[0]
    for y in outs:
        st = _call(lib, "ndconv_conv_fft_noalloc", p, x, k, y)
        assert st == 0, _abi.last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert pool.high() == 0
    ref = y_ref.cpu().numpy()
    for y in outs:
        assert normwise_err(y.cpu().numpy(), ref) <= TOL32
    if name == "2d_f32":
        # and against the f64 oracle itself
        xn, kn = x.cpu().numpy().astype(np.float64), k.cpu().numpy().astype(np.float64)
        st, y64 = O.conv_fft(problem(F64, xn, with_dilation(kn, dil), mode, pm), xn, kn, 4)
        assert st == 0
        assert normwise_err(outs[1].cpu().numpy(), y64) <= TOL32


def test_noalloc_rejects_oversize(lib):
    import torch
    from ndconv import _abi, build_problem
    xs = (1024, 4096)  # spectra far above 16 MiB
    x = torch.zeros(xs, device="cuda")
    k = torch.zeros((3, 3), device="cuda")
    y = torch.zeros(xs, device="cuda")
    p = build_problem(_abi.F32, xs, with_dilation(k, 1), ConvMode.Same, PaddingMode.Zeros)
    st = _call(lib, "ndconv_conv_fft_noalloc", p, x, k, y)
    assert st == _abi.ERR_NO_MEMORY
    assert "16 MiB" in _abi.last_error()


def test_noalloc_unsupported_where_conv_fft_runs_direct(lib):
    """A kernel row longer than the longest overlap-save segment: no FFT form
    applies.  ndconv_conv_fft takes the direct kernels; the allocation-free
    entry point reports NDCONV_ERR_UNSUPPORTED and leaves the output alone."""
    import torch
    from ndconv import _abi, build_problem
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand((70000,), generator=g, device="cuda")
    k = torch.rand((30001,), generator=g, device="cuda")
    p = build_problem(_abi.F32, (70000,), with_dilation(k, 1), ConvMode.Same, PaddingMode.Zeros)
    y_ref = torch.empty((70000,), device="cuda")
    assert _call(lib, "ndconv_conv_fft", p, x, k, y_ref, None) == 0, _abi.last_error()
    y = torch.full((70000,), 7.0, device="cuda")
    st = _call(lib, "ndconv_conv_fft_noalloc", p, x, k, y)
    assert st == _abi.ERR_UNSUPPORTED
    torch.cuda.synchronize()
    assert bool((y == 7.0).all())
    assert torch.isfinite(y_ref).all()
