"""The 3xBF16 split tensor-core direct path (tcgen05 + TMA) against the f64
oracle: normwise error <= 1e-5 on f32 problems, the reference's NaN
pattern when an input is not finite, and UNSUPPORTED where it does not
apply."""
import numpy as np
import pytest

import ndconv
from ndconv import _abi
from helpers import F64, BorderType, ConvMode, PaddingMode, normwise_err, problem, with_dilation
from oracle import oracle as O
from test_gpu_parity import _c3, _oracle64

pytestmark = pytest.mark.gpu
TOL32 = 1e-5
BF = _abi.ALGO_DIRECT_BF16X3


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()


@pytest.mark.parametrize("shape,kshape,dil,mode,pm", [
    ((40, 150), (3, 5), 1, ConvMode.Same, PaddingMode.Zeros),
    ((70, 300), (7, 15), 2, ConvMode.Same, PaddingMode.Custom([BorderType.Reflect, BorderType.Circular])),
    ((3, 70, 150), (2, 3, 5), [1, 2, 3], ConvMode.Custom([1, 2, 3], [2, 1, 2]), PaddingMode.Replicate),
    ((5, 9, 140), (2, 3, 4), 1, ConvMode.Explicit([[1, 0], [2, 1], [0, 3]], [2, 1, 3]), PaddingMode.Const(0.5)),
    ((1000,), (31,), 1, ConvMode.Full, PaddingMode.Zeros),
    ((130, 257), (17, 17), 1, ConvMode.Valid, PaddingMode.Zeros),
    ((64, 640), (15, 63), 1, ConvMode.Same, PaddingMode.Circular),
    # strides along the middle axis, kernels of several row groups, dilation
    # that shrinks the row groups, rows of one output
    ((90, 300), (5, 9), [3, 2], ConvMode.Custom([3, 2], [3, 2]), PaddingMode.Reflect),
    ((300, 200), (40, 21), 1, ConvMode.Same, PaddingMode.Zeros),
    ((260, 180), (9, 7), [30, 1], ConvMode.Same, PaddingMode.Replicate),
    ((4, 260, 90), (3, 33, 5), [2, 1, 3], ConvMode.Custom([2, 5, 1], [1, 3, 2]), PaddingMode.Zeros),
    ((1, 4000), (1, 127), 1, ConvMode.Valid, PaddingMode.Zeros),
    # one kernel row per group (row dilation 70) in several groups, and a
    # kernel of one row: the epilogue reads TMEM rows as output rows
    ((300, 120), (3, 7), [70, 1], ConvMode.Same, PaddingMode.Reflect),
    ((200, 333), (1, 45), 1, ConvMode.Full, PaddingMode.Replicate),
])
def test_bf16x3_vs_oracle(shape, kshape, dil, mode, pm):
    rng = np.random.default_rng(sum(shape) + sum(kshape))
    x = rng.random(shape).astype(np.float32)
    k = rng.random(kshape).astype(np.float32)
    y64 = _oracle64(x, with_dilation(k, dil), mode, pm)
    y = ndconv.conv_algo(x, with_dilation(k, dil), mode, pm, BF)
    assert y.shape == y64.shape
    assert normwise_err(y, y64) <= TOL32, normwise_err(y, y64)
    # signed data (cancellation) too
    xs, ks = (x - 0.5).astype(np.float32), (k - 0.5).astype(np.float32)
    y64 = _oracle64(xs, with_dilation(ks, dil), mode, pm)
    assert normwise_err(ndconv.conv_algo(xs, with_dilation(ks, dil), mode, pm, BF), y64) <= TOL32


@pytest.mark.parametrize("cplx", [False])
def test_bf16x3_3d_case(cplx):
    x, kw, mode, pm = _c3(cplx)
    y64 = _oracle64(x, kw, mode, pm)
    assert normwise_err(ndconv.conv_algo(x, kw, mode, pm, BF), y64) <= TOL32


def test_bf16x3_nonfinite_follows_reference():
    rng = np.random.default_rng(3)
    x = rng.random((20, 200)).astype(np.float32)
    k = rng.random((5, 9)).astype(np.float32)
    x[7, 33] = np.inf
    mode, pm = ConvMode.Same, PaddingMode.Zeros
    st, y64 = O.conv(problem(F64, x, k, mode, pm), x.astype(np.float64), k.astype(np.float64))
    y = ndconv.conv_algo(x, k, mode, pm, BF)
    assert np.array_equal(np.isnan(y), np.isnan(y64)) and np.array_equal(np.isinf(y), np.isinf(y64))
    fin = np.isfinite(y64)
    assert np.allclose(y[fin], y64[fin], rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("bn", [16, 32, 64])
def test_bf16x3_tile_widths_agree(bn):
    """Every tile width the tuner may pick meets the same bound."""
    rng = np.random.default_rng(bn)
    x = rng.random((150, 333)).astype(np.float32) - 0.5
    k = rng.random((3, 19)).astype(np.float32) - 0.5
    mode, pm = ConvMode.Same, PaddingMode.Custom([BorderType.Circular, BorderType.Reflect])
    y64 = _oracle64(x, k, mode, pm)
    L = _abi.lib()
    old = L.ndconv_get_tuning(_abi.TUNE_BF16X3_BN)
    try:
        assert L.ndconv_set_tuning(_abi.TUNE_BF16X3_BN, bn) == 0
        assert normwise_err(ndconv.conv_algo(x, k, mode, pm, BF), y64) <= TOL32
    finally:
        L.ndconv_set_tuning(_abi.TUNE_BF16X3_BN, old)


def test_bf16x3_unsupported():
    x = np.ones((30, 40), np.float32)
    with pytest.raises(ndconv.ConvError):
        ndconv.conv_algo(x.astype(np.float64), np.ones((3, 3)), ConvMode.Same, PaddingMode.Zeros, BF)
    with pytest.raises(ndconv.ConvError):
        ndconv.conv_algo(x.astype(np.int32), np.ones((3, 3), np.int32), ConvMode.Same, PaddingMode.Zeros, BF)


@pytest.mark.parametrize("shape,kshape,dil,mode,pm,n", [
    ((60, 170), (9, 13), [1, 2], ConvMode.Same, PaddingMode.Custom([BorderType.Reflect, BorderType.Circular]), 5),
    ((3, 40, 90), (2, 7, 11), 1, ConvMode.Same, PaddingMode.Zeros, 4),
    ((150, 130), (21, 5), 1, ConvMode.Valid, PaddingMode.Zeros, 3),
    ((40, 70), (3, 3), 1, ConvMode.Full, PaddingMode.Replicate, 7),
])
def test_bf16x3_batch_equals_single_calls(shape, kshape, dil, mode, pm, n):
    """ndconv_conv_bf16x3_batch: each instance bit for bit its single call,
    and within 1e-5 of the f64 oracle."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(sum(shape) + n)
    xs = [torch.rand(shape, generator=g, device="cuda") - 0.5 for _ in range(n)]
    ks = [torch.rand(kshape, generator=g, device="cuda") - 0.5 for _ in range(n)]
    ys = ndconv.conv_bf16x3_batch(xs, [with_dilation(k, dil) for k in ks], mode, pm)
    for i in range(n):
        y1 = ndconv.conv_algo(xs[i], with_dilation(ks[i], dil), mode, pm, BF)
        assert torch.equal(ys[i], y1), i
    i = n - 1
    y64 = _oracle64(xs[i].cpu().numpy(), with_dilation(ks[i].cpu().numpy(), dil), mode, pm)
    assert normwise_err(ys[i].cpu().numpy(), y64) <= TOL32


def test_bf16x3_batch_nonfinite_instance():
    """A non-finite value in one instance: every instance through the FP32
    loop, with the reference's NaN pattern where the values are not finite."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(11)
    xs = [torch.rand((20, 100), generator=g, device="cuda") for _ in range(3)]
    ks = [torch.rand((5, 9), generator=g, device="cuda") for _ in range(3)]
    xs[1][4, 17] = float("nan")
    mode, pm = ConvMode.Same, PaddingMode.Zeros
    ys = ndconv.conv_bf16x3_batch(xs, ks, mode, pm)
    for i in range(3):
        x, k = xs[i].cpu().numpy(), ks[i].cpu().numpy()
        st, y64 = O.conv(problem(F64, x, k, mode, pm), x.astype(np.float64), k.astype(np.float64))
        y = ys[i].cpu().numpy()
        assert np.array_equal(np.isnan(y), np.isnan(y64))
        fin = np.isfinite(y64)
        assert np.allclose(y[fin], y64[fin], rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("shape,kshape,dil,mode,pm", [
    ((10, 100, 200), (5, 11, 31), 1, ConvMode.Same, PaddingMode.Zeros),
    ((70, 180), (9, 17), [2, 1], ConvMode.Same, PaddingMode.Const(complex(0.5, -1.25))),
    ((40, 90), (5, 7), 1, ConvMode.Custom([2, 3], [1, 2]),
     PaddingMode.Custom([BorderType.Reflect, BorderType.Const(complex(-0.75, 2.0))])),
    ((600,), (33,), 1, ConvMode.Full, PaddingMode.Circular),
])
def test_bf16x3_complex_vs_oracle(shape, kshape, dil, mode, pm):
    """Complex<f32> on the tensor cores (four real 3xBF16 convolutions over
    the interleaved parts): within 1e-5 normwise of the f64 oracle, border
    constants with imaginary parts included."""
    rng = np.random.default_rng(sum(shape) + 7)
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    k = (rng.standard_normal(kshape) + 1j * rng.standard_normal(kshape)).astype(np.complex64)
    y64 = _oracle64(x, with_dilation(k, dil), mode, pm)
    y = ndconv.conv_algo(x, with_dilation(k, dil), mode, pm, BF)
    assert y.shape == y64.shape
    assert normwise_err(y, y64) <= TOL32, normwise_err(y, y64)


def test_bf16x3_complex_strided_view():
    """A strided complex view (every other column) is read in place."""
    import torch
    rng = np.random.default_rng(5)
    base = (rng.standard_normal((50, 160)) + 1j * rng.standard_normal((50, 160))).astype(np.complex64)
    k = (rng.standard_normal((7, 9)) + 1j * rng.standard_normal((7, 9))).astype(np.complex64)
    xv = torch.from_numpy(base).cuda()[:, ::2]
    mode, pm = ConvMode.Same, PaddingMode.Replicate
    y = ndconv.conv_algo(xv, torch.from_numpy(k).cuda(), mode, pm, BF).cpu().numpy()
    y64 = _oracle64(np.ascontiguousarray(base[:, ::2]), k, mode, pm)
    assert normwise_err(y, y64) <= TOL32


def _fold_of(x, k, mode, pm):
    """(S, R) of the tile plan: outputs per virtual row and virtual rows of a
    folded single row, (0, 1) when the row is not folded."""
    import ctypes
    p = problem(_abi.F32, x, k, mode, pm)
    out = (ctypes.c_int64 * 18)()
    assert _abi.lib().ndconv_bf16x3_plan(ctypes.byref(p), out) == 0, _abi.last_error()
    return int(out[16]), int(out[17])


@pytest.mark.parametrize("shape,kshape,dil,mode,pm", [
    ((200000,), (255,), 1, ConvMode.Same, PaddingMode.Reflect),
    ((50000,), (31,), 2, ConvMode.Custom([7], [3]), PaddingMode.Circular),
    ((30000,), (17,), 3, ConvMode.Explicit([[5, 40]], [2]), PaddingMode.Replicate),
    ((611,), (31,), 1, ConvMode.Full, PaddingMode.Zeros),        # last virtual row: one output
    ((5000,), (3,), 1, ConvMode.Same, PaddingMode.Zeros),        # S = BN
    ((9000,), (63,), 1, ConvMode.Same, PaddingMode.Const(0.5)),
    ((1, 20000), (1, 101), [1, 2], ConvMode.Same, PaddingMode.Custom([BorderType.Zeros, BorderType.Reflect])),
    ((100000,), (1001,), 1, ConvMode.Valid, PaddingMode.Zeros),
])
def test_bf16x3_folded_row_vs_oracle(shape, kshape, dil, mode, pm):
    """A single row cut into stretches that fill the 128 accumulator lanes:
    within 1e-5 normwise of the f64 oracle, every output written once (the
    output buffer starts as NaN)."""
    import torch
    rng = np.random.default_rng(sum(shape) + sum(kshape))
    x = rng.random(shape).astype(np.float32) - 0.5
    k = rng.random(kshape).astype(np.float32) - 0.5
    kw = with_dilation(k, dil)
    S, R = _fold_of(x, kw, mode, pm)
    assert S > 0 and R >= 2
    y64 = _oracle64(x, kw, mode, pm)
    import ctypes
    xd, kd = torch.from_numpy(x).cuda(), torch.from_numpy(k).cuda()
    yd = torch.full(y64.shape, float("nan"), device="cuda")
    p = problem(_abi.F32, x, kw, mode, pm)
    st = _abi.lib().ndconv_conv_algo(ctypes.byref(p), BF, ctypes.c_void_p(xd.data_ptr()),
                                     ctypes.c_void_p(kd.data_ptr()), ctypes.c_void_p(yd.data_ptr()),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, _abi.last_error()
    y = yd.cpu().numpy()
    assert np.isfinite(y).all()
    assert normwise_err(y, y64) <= TOL32, normwise_err(y, y64)


@pytest.mark.parametrize("bn", [16, 32, 64])
def test_bf16x3_folded_row_tile_widths(bn):
    """Each tile width folds the row into its own stretch length."""
    rng = np.random.default_rng(40 + bn)
    x = rng.random((33333,)).astype(np.float32) - 0.5
    k = rng.random((45,)).astype(np.float32) - 0.5
    mode, pm = ConvMode.Full, PaddingMode.Reflect
    y64 = _oracle64(x, k, mode, pm)
    L = _abi.lib()
    old = L.ndconv_get_tuning(_abi.TUNE_BF16X3_BN)
    try:
        assert L.ndconv_set_tuning(_abi.TUNE_BF16X3_BN, bn) == 0
        S, R = _fold_of(x, k, mode, pm)
        assert S % bn == 0 and R >= 2
        assert normwise_err(ndconv.conv_algo(x, k, mode, pm, BF), y64) <= TOL32
    finally:
        L.ndconv_set_tuning(_abi.TUNE_BF16X3_BN, old)


def test_bf16x3_folded_row_nonfinite():
    """A non-finite sample in a folded row: the FP32 loop over the virtual
    rows gives the reference's NaN pattern."""
    rng = np.random.default_rng(12)
    x = rng.random((7000,)).astype(np.float32)
    k = rng.random((31,)).astype(np.float32)
    x[4321] = np.inf
    mode, pm = ConvMode.Full, PaddingMode.Zeros
    assert _fold_of(x, k, mode, pm)[1] >= 2
    st, y64 = O.conv(problem(F64, x, k, mode, pm), x.astype(np.float64), k.astype(np.float64))
    y = ndconv.conv_algo(x, k, mode, pm, BF)
    assert np.array_equal(np.isnan(y), np.isnan(y64)) and np.array_equal(np.isinf(y), np.isinf(y64))
    fin = np.isfinite(y64)
    assert np.allclose(y[fin], y64[fin], rtol=1e-5, atol=1e-5)


def test_bf16x3_folded_row_batch_and_complex():
    """Folded rows in a batch (bit for bit the single calls) and in the
    complex form's four real views."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(21)
    mode, pm = ConvMode.Same, PaddingMode.Circular
    xs = [torch.rand((12345,), generator=g, device="cuda") - 0.5 for _ in range(6)]
    ks = [torch.rand((37,), generator=g, device="cuda") - 0.5 for _ in range(6)]
    ys = ndconv.conv_bf16x3_batch(xs, ks, mode, pm)
    for i in range(6):
        assert torch.equal(ys[i], ndconv.conv_algo(xs[i], ks[i], mode, pm, BF)), i
    y64 = _oracle64(xs[5].cpu().numpy(), ks[5].cpu().numpy(), mode, pm)
    assert normwise_err(ys[5].cpu().numpy(), y64) <= TOL32
    rng = np.random.default_rng(22)
    x = (rng.standard_normal(20000) + 1j * rng.standard_normal(20000)).astype(np.complex64)
    k = (rng.standard_normal(63) + 1j * rng.standard_normal(63)).astype(np.complex64)
    y64 = _oracle64(x, k, ConvMode.Full, PaddingMode.Reflect)
    assert normwise_err(ndconv.conv_algo(x, k, ConvMode.Full, PaddingMode.Reflect, BF), y64) <= TOL32
