"""Rows longer than one CTA's shared memory on the FFT path: overlap-save
segments of the contiguous axis (row-spectral form for 2-D / 3-D, fused rows
for 1-D), against the f64 oracle at normwise error <= 1e-5, for every element
type, strides, dilation, border modes and no_reverse; the full N-d form
reports UNSUPPORTED for such rows instead of running."""
import numpy as np
import pytest

import ndconv
from ndconv import _abi
from helpers import BorderType, ConvMode, PaddingMode, normwise_err, with_dilation
from test_gpu_parity import _oracle64

pytestmark = pytest.mark.gpu
TOL32 = 1e-5
TOL64 = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()


def _data(rng, shape, dtype):
    if np.dtype(dtype).kind == "c":
        return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)
    return rng.random(shape).astype(dtype)


CASES = [
    # shape, kernel, dilation, mode, padding, dtype
    ((200_000,), (31,), 1, ConvMode.Full, PaddingMode.Zeros, np.float32),
    ((100_000,), (2_501,), 2, ConvMode.Same, PaddingMode.Reflect, np.float32),
    ((60_001,), (77,), 1, ConvMode.Custom([0], [3]), PaddingMode.Circular, np.float32),
    ((3, 60_000), (3, 101), 2, ConvMode.Same, PaddingMode.Custom([BorderType.Reflect, BorderType.Circular]),
     np.float32),
    ((4, 40_000), (2, 15), 1, ConvMode.Custom([1, 2], [2, 3]), PaddingMode.Replicate, np.float32),
    ((2, 3, 30_000), (2, 2, 21), [1, 2, 3], ConvMode.Valid, PaddingMode.Zeros, np.float32),
    ((30_000,), (77,), 1, ConvMode.Valid, PaddingMode.Zeros, np.complex64),
    ((2, 20_000), (3, 33), 1, ConvMode.Same, PaddingMode.Const(0.5), np.complex64),
    ((40_000,), (301,), 1, ConvMode.Same, PaddingMode.Replicate, np.float64),
    ((20_000,), (65,), 2, ConvMode.Full, PaddingMode.Zeros, np.complex128),
    ((60_000,), (15_001,), 1, ConvMode.Same, PaddingMode.Zeros, np.float32),  # kernel near the segment limit
]


@pytest.mark.parametrize("shape,kshape,dil,mode,pm,dt", CASES)
@pytest.mark.parametrize("reverse", [True, False])
def test_long_rows_fft_vs_oracle(shape, kshape, dil, mode, pm, dt, reverse):
    rng = np.random.default_rng(sum(shape) + sum(kshape))
    x = _data(rng, shape, dt)
    k = _data(rng, kshape, dt)
    kw = with_dilation(k, dil)
    if not reverse:
        kw = kw.no_reverse()
    y64 = _oracle64(x, kw, mode, pm)
    tol = TOL32 if np.dtype(dt) in (np.float32, np.complex64) else TOL64
    for algo in (_abi.ALGO_FFT, _abi.ALGO_FFT_RS, _abi.ALGO_FFT_RS_POW2):
        y = ndconv.conv_algo(x, kw, mode, pm, algo)
        assert y.shape == y64.shape
        assert normwise_err(y, y64) <= tol, (algo, normwise_err(y, y64))
    for algo in (_abi.ALGO_FFT_ND, _abi.ALGO_FFT_ND_POW2):
        with pytest.raises(ndconv.ConvError):
            ndconv.conv_algo(x, kw, mode, pm, algo)


def test_long_leading_axis():
    # 40,000-long leading axis: too long for one column pass of the N-d form
    # (reported); the row-spectral form transforms rows only; conv_fft runs
    # the direct kernels for it
    rng = np.random.default_rng(9)
    x = rng.random((40_000, 3)).astype(np.float32)
    k = rng.random((101, 3)).astype(np.float32)
    mode, pm = ConvMode.Same, PaddingMode.Reflect
    y64 = _oracle64(x, k, mode, pm)
    assert normwise_err(ndconv.conv_algo(x, k, mode, pm, _abi.ALGO_FFT_RS), y64) <= TOL32
    assert normwise_err(ndconv.conv_fft(x, k, mode, pm), y64) <= TOL32
    with pytest.raises(ndconv.ConvError):
        ndconv.conv_algo(x, k, mode, pm, _abi.ALGO_FFT_ND)


def test_long_rows_processor_and_batch():
    import torch
    from ndconv.batch import BatchPlan
    rng = np.random.default_rng(11)
    shapes = [((150_000,), (63,)), ((2, 50_000), (3, 41)), ((300, 400), (5, 7))]
    xs = [torch.from_numpy(rng.random(s).astype(np.float32)).cuda() for s, _ in shapes]
    ks = [torch.from_numpy(rng.random(k).astype(np.float32)).cuda() for _, k in shapes]
    modes = [(ConvMode.Same, PaddingMode.Circular)] * len(shapes)
    plan = BatchPlan(modes, xs, ks, algos=[1] * len(shapes))
    assert plan.info()["n_standalone"] == 0
    plan.run(graph=True)
    plan.check()
    torch.cuda.synchronize()
    proc = ndconv.get_fft_processor(torch.float32)
    for i in range(len(shapes)):
        y64 = _oracle64(xs[i].cpu().numpy(), ks[i].cpu().numpy(), *modes[i])
        assert normwise_err(plan.outs[i].cpu().numpy(), y64) <= TOL32, i
        # the processor path (reused workspace) gives the same result class
        yp = ndconv.conv_fft_with_processor(xs[i], ks[i], *modes[i], proc)
        assert normwise_err(yp.cpu().numpy(), y64) <= TOL32, i
    plan.close()


def test_kernel_row_beyond_segments_falls_back():
    # a 7,001-tap complex f64 kernel row is longer than any segment a CTA
    # holds: the explicit FFT forms report it, conv_fft runs the direct kernels
    rng = np.random.default_rng(13)
    x = _data(rng, (10_000,), np.complex128)
    k = _data(rng, (7_001,), np.complex128)
    mode, pm = ConvMode.Same, PaddingMode.Zeros
    y64 = _oracle64(x, k, mode, pm)
    with pytest.raises(ndconv.ConvError):
        ndconv.conv_algo(x, k, mode, pm, _abi.ALGO_FFT_RS)
    assert normwise_err(ndconv.conv_fft(x, k, mode, pm), y64) <= TOL64


def test_long_rows_strided_view():
    # every other sample of a 120,000-sample row, read in place through its stride
    import torch
    g = torch.Generator(device="cuda").manual_seed(17)
    base = torch.rand((3, 120_000), generator=g, device="cuda")
    x = base[:, ::2]
    k = torch.rand((2, 45), generator=g, device="cuda")
    mode, pm = ConvMode.Same, PaddingMode.Custom([BorderType.Replicate, BorderType.Reflect])
    y64 = _oracle64(x.contiguous().cpu().numpy(), k.cpu().numpy(), mode, pm)
    for algo in (_abi.ALGO_FFT, _abi.ALGO_FFT_RS):
        y = ndconv.conv_algo(x, k, mode, pm, algo)
        assert normwise_err(y.cpu().numpy(), y64) <= TOL32, algo
