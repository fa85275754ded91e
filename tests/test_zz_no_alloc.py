"""ndconv_conv_fft_noalloc: FFT convolution for callers that cannot allocate.

Real-time hosts that forbid device allocation after start-up, and plugins
whose host application owns every allocation, cannot let the library call
cudaMalloc.  This entry point uses a fixed 16 MiB device array
inside the library instead.  Its results must match ndconv_conv_fft (the
allocating entry point) within the tests' f32 tolerance, on two calls in a
row (the array keeps the previous call's contents), and oversize problems
must be rejected.  Collected last so a failure here leaves every other test
already run; passes alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

from helpers import BorderType, ConvMode, PaddingMode, normwise_err, with_dilation

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
    outs = []
    for _ in range(2):
        y = torch.full(shape, float("nan"), device="cuda", dtype=tdt)
        st = _call(lib, "ndconv_conv_fft_noalloc", p, x, k, y)
        assert st == 0, _abi.last_error()
        outs.append(y)
    torch.cuda.synchronize()
    ref = y_ref.cpu().numpy()
    for y in outs:
        assert normwise_err(y.cpu().numpy(), ref) <= TOL32


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
