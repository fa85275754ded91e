"""The 8- to 64-bit integer element types of ConvExt::conv on the GPU.

The crate's conv is generic over T: NumAssign + Copy (src/conv/mod.rs:78-83,
118-124); release-mode Rust wraps, so its sums are modulo 2^bits.  For u8,
i8, u16, i16, u32, i64 and u64 the library must equal the oracle bit for bit
on random 1-3-D problems (every convolution mode, every border kind with
integral constants, dilation, stride, reversed and unreversed kernels,
values spread over the whole range so products overflow), on a larger 2-D
case that takes the row-blocked sliding-window kernel, and on strided views
(the narrow types are widened on the device through the view's strides).
The crate's u8 circular-padding literal (src/padding/mod.rs:619-624) is
re-asserted through a one-tap kernel; the FFT and batch entry points refuse
these types.
"""
import numpy as np
import pytest

import ndconv
from ndconv import _abi
from helpers import BorderType, ConvMode, PaddingMode, problem, with_dilation
from oracle import oracle as O
from test_gpu_parity import _kw, random_case

pytestmark = pytest.mark.gpu

TYPES = [(_abi.U8, np.uint8), (_abi.I8, np.int8), (_abi.U16, np.uint16), (_abi.I16, np.int16),
         (_abi.U32, np.uint32), (_abi.I64, np.int64), (_abi.U64, np.uint64)]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()


def _values(rng, shape, npt):
    info = np.iinfo(npt)
    # 64-bit values stay within the oracle's exact range (|v| <= 2^53)
    hi, lo = min(int(info.max), 1 << 50), max(int(info.min), -(1 << 50))
    return rng.integers(lo, hi, shape, dtype=np.int64, endpoint=True).astype(npt)


def _int_pm(pm, c):
    fix = lambda b: BorderType.Const(c) if b.kind == _abi.BORDER_CONST else b  # noqa: E731
    if pm.kind == _abi.PAD_CONST:
        return PaddingMode.Const(c)
    if pm.kind == _abi.PAD_CUSTOM:
        return PaddingMode.Custom([fix(b) for b in pm.borders])
    if pm.kind == _abi.PAD_EXPLICIT:
        return PaddingMode.Explicit([[fix(b) for b in bb] for bb in pm.borders])
    return pm


def _check(code, npt, x, k, kw, mode, pm):
    st, yo = O.conv(problem(code, x, kw, mode, pm), x, k)
    if st:
        with pytest.raises(ndconv.ConvError):
            ndconv.conv(x, kw, mode, pm)
        return False
    y = ndconv.conv(x, kw, mode, pm)
    assert y.dtype == npt
    assert np.array_equal(y, yo), (npt, x.shape, k.shape, mode, pm)
    return True


@pytest.mark.parametrize("code,npt", TYPES)
def test_random_problems_bit_exact(code, npt):
    rng = np.random.default_rng(900 + code)
    n_ok = 0
    for trial in range(24):
        shape, kshape, kw0, mode, pm = random_case(rng, 1 + trial % 3)
        c = int(rng.integers(0, 200)) if np.iinfo(npt).min == 0 else int(rng.integers(-100, 100))
        pm = _int_pm(pm, c)
        x, k = _values(rng, shape, npt), _values(rng, kshape, npt)
        k.flat[::5] = 0  # zero taps are skipped like gen_offset_list (src/dilation/mod.rs:47-50)
        n_ok += _check(code, npt, x, k, _kw(kw0, k), mode, pm)
    assert n_ok >= 12


@pytest.mark.parametrize("code,npt", TYPES)
def test_sliding_window_case_bit_exact(code, npt):
    rng = np.random.default_rng(950 + code)
    x, k = _values(rng, (70, 333), npt), _values(rng, (5, 9), npt)
    mode = ConvMode.Explicit([[4, 4], [8, 8]], [1, 1])
    for pm in (PaddingMode.Reflect, PaddingMode.Custom([BorderType.Const(7), BorderType.Circular])):
        assert _check(code, npt, x, k, with_dilation(k, [2, 2]), mode, pm)


@pytest.mark.parametrize("npt", [np.uint8, np.int8, np.int16, np.int64])
def test_strided_views(npt):
    import torch
    code = dict((t, c) for c, t in TYPES)[npt]
    rng = np.random.default_rng(3)
    base = _values(rng, (20, 2 * 37), npt)
    kb = _values(rng, (3, 2 * 5), npt)
    xv = torch.from_numpy(base).cuda()[:, ::2]  # a view with column stride 2
    kv = torch.from_numpy(kb).cuda()[:, 1::2]
    x, k = base[:, ::2].copy(), kb[:, 1::2].copy()
    mode, pm = ConvMode.Same, PaddingMode.Replicate
    st, yo = O.conv(problem(code, x, k, mode, pm), x, k)
    assert st == 0
    y = ndconv.conv(xv, with_dilation(kv, 1), mode, pm)
    assert np.array_equal(y.cpu().numpy(), yo)


def test_u8_circular_padding_literal():
    """src/padding/mod.rs:619-624: [1u8, 2, 3] padded circularly by one
    sample each side is [3, 1, 2, 3, 1]."""
    x, k = np.array([1, 2, 3], np.uint8), np.array([1], np.uint8)
    y = ndconv.conv(x, with_dilation(k, 1), ConvMode.Explicit([[1, 1]], [1]), PaddingMode.Circular)
    assert y.dtype == np.uint8 and y.tolist() == [3, 1, 2, 3, 1]


def test_other_entry_points_refuse():
    import torch
    x = np.arange(12, dtype=np.uint8).reshape(3, 4)
    k = np.ones((2, 2), np.uint8)
    with pytest.raises(ndconv.ConvError):
        ndconv.conv_fft(x, with_dilation(k, 1), ConvMode.Same, PaddingMode.Zeros)
    xs = [torch.zeros((3, 4), dtype=torch.int64, device="cuda") for _ in range(2)]
    ks = [torch.ones((2, 2), dtype=torch.int64, device="cuda") for _ in range(2)]
    with pytest.raises(ndconv.ConvError):
        ndconv.conv_batch(xs, [with_dilation(kk, 1) for kk in ks], ConvMode.Same, PaddingMode.Zeros)
