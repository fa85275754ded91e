"""Kernel-spectrum reuse through the processor ("baked" kernel): results
are identical to fresh conv_fft calls, and the baked spectrum is used only
for the same geometry and the same kernel tensor."""
import numpy as np
import pytest

import ndconv
from helpers import BorderType, ConvMode, PaddingMode, with_dilation

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()


@pytest.mark.parametrize("shape,kshape,dil,mode,pm,dt", [
    ((200, 5000), (11, 31), 2, ConvMode.Same, PaddingMode.Custom([BorderType.Reflect, BorderType.Circular]),
     "float32"),
    ((10, 100, 200), (5, 11, 31), 1, ConvMode.Same, PaddingMode.Zeros, "float32"),
    ((60, 70), (41, 9), 1, ConvMode.Full, PaddingMode.Replicate, "float64"),
    ((5000,), (31,), 1, ConvMode.Full, PaddingMode.Zeros, "float32"),
    ((6, 30, 40), (3, 4, 5), 1, ConvMode.Valid, PaddingMode.Zeros, "complex64"),
])
def test_baked_equals_fresh(shape, kshape, dil, mode, pm, dt):
    import torch
    tdt = getattr(torch, dt)
    g = torch.Generator(device="cuda").manual_seed(11)
    mk = (lambda s: torch.randn(s, generator=g, device="cuda", dtype=tdt)) if tdt.is_complex else \
        (lambda s: torch.rand(s, generator=g, device="cuda", dtype=tdt))
    k = mk(kshape)
    proc = ndconv.get_fft_processor(tdt)
    x0 = mk(shape)
    proc.bake(x0, with_dilation(k, dil), mode, pm)
    for _ in range(3):
        x = mk(shape)
        y = ndconv.conv_fft_with_processor(x, with_dilation(k, dil), mode, pm, proc)
        assert torch.equal(y, ndconv.conv_fft(x, with_dilation(k, dil), mode, pm))
    # another kernel tensor of the same geometry: not the baked one
    k2 = mk(kshape)
    y2 = ndconv.conv_fft_with_processor(x, with_dilation(k2, dil), mode, pm, proc)
    assert torch.equal(y2, ndconv.conv_fft(x, with_dilation(k2, dil), mode, pm))
    proc.close()


def test_baked_ignored_for_other_geometry():
    import torch
    k = torch.rand((5, 9), device="cuda")
    proc = ndconv.get_fft_processor(torch.float32)
    proc.bake(torch.empty((40, 300), device="cuda"), k, ConvMode.Same, PaddingMode.Zeros)
    x = torch.rand((41, 300), device="cuda")  # different data shape
    y = ndconv.conv_fft_with_processor(x, k, ConvMode.Same, PaddingMode.Zeros, proc)
    assert torch.equal(y, ndconv.conv_fft(x, k, ConvMode.Same, PaddingMode.Zeros))
    x = torch.rand((40, 300), device="cuda")
    y = ndconv.conv_fft_with_processor(x, k, ConvMode.Full, PaddingMode.Zeros, proc)  # different mode
    assert torch.equal(y, ndconv.conv_fft(x, k, ConvMode.Full, PaddingMode.Zeros))
    proc.close()
