"""Large sizes through the C ABI, where the f64 oracle would take too long:
size-independent properties instead (FFT forms agree with the direct path,
linearity, shift equivariance), plus one long 1-D row against the oracle."""
import numpy as np
import pytest

import ndconv
from ndconv import _abi
from helpers import F64, BorderType, ConvMode, PaddingMode, normwise_err, problem, with_dilation
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()


def test_long_row_against_oracle():
    # 1,000,000-sample row: longer than one CTA's shared memory, so conv_fft
    # takes the direct kernels; both must match the f64 oracle
    rng = np.random.default_rng(1)
    x = rng.random(1_000_000).astype(np.float32)
    k = rng.random(31).astype(np.float32)
    mode, pm = ConvMode.Full, PaddingMode.Zeros
    st, y64 = O.conv(problem(F64, x, k, mode, pm), x.astype(np.float64), k.astype(np.float64))
    assert st == 0
    assert normwise_err(ndconv.conv(x, k, mode, pm), y64) <= 1e-5
    assert normwise_err(ndconv.conv_fft(x, k, mode, pm), y64) <= 1e-5


@pytest.mark.parametrize("shape,kshape,dil,pm", [
    ((2048, 2048), (31, 31), 1, PaddingMode.Zeros),
    ((1024, 4096), (15, 63), 2, PaddingMode.Custom([BorderType.Reflect, BorderType.Circular])),
    ((64, 256, 256), (5, 9, 9), 1, PaddingMode.Replicate),
])
def test_large_fft_forms_agree_with_direct(shape, kshape, dil, pm):
    import torch
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand(shape, generator=g, device="cuda")
    k = torch.rand(kshape, generator=g, device="cuda")
    mode = ConvMode.Same
    yd = ndconv.conv(x, with_dilation(k, dil), mode, pm).double()
    for algo in (_abi.ALGO_FFT, _abi.ALGO_FFT_ND, _abi.ALGO_FFT_RS, _abi.ALGO_FFT_RS_POW2):
        try:
            yf = ndconv.conv_algo(x, with_dilation(k, dil), mode, pm, algo).double()
        except ndconv.ConvError:
            continue  # a form whose transforms do not fit (reported, not silently wrong)
        err = float(torch.linalg.vector_norm(yf - yd) / torch.linalg.vector_norm(yd))
        assert err <= 2e-5, (algo, err)


def test_linearity_and_shift_large():
    import torch
    g = torch.Generator(device="cuda").manual_seed(5)
    shape, k = (512, 4096), torch.rand((11, 31), generator=g, device="cuda")
    x1 = torch.rand(shape, generator=g, device="cuda")
    x2 = torch.rand(shape, generator=g, device="cuda")
    mode, pm = ConvMode.Full, PaddingMode.Zeros
    for f in (ndconv.conv, ndconv.conv_fft):
        y1, y2 = f(x1, k, mode, pm).double(), f(x2, k, mode, pm).double()
        y12 = f(2.0 * x1 - 0.5 * x2, k, mode, pm).double()
        ref = 2.0 * y1 - 0.5 * y2
        assert float(torch.linalg.vector_norm(y12 - ref) / torch.linalg.vector_norm(ref)) <= 2e-5
    # Full mode with zero padding is shift-equivariant along the contiguous axis
    xs = torch.zeros_like(x1)
    xs[:, 7:] = x1[:, :-7]
    ya, yb = ndconv.conv(x1, k, mode, pm), ndconv.conv(xs, k, mode, pm)
    assert torch.allclose(yb[:, 7:7 + 4000], ya[:, :4000], rtol=1e-5, atol=1e-5)
