"""The oracle's integer convolutions (ConvExt::conv, src/conv/mod.rs:170-197)
for the 8- to 64-bit element types, pinned on the host.

Release-mode Rust wraps integer overflow, so the crate's sums are the sums
of products modulo 2^bits.  The oracle accumulates in wrapping u64 and keeps
the low bits; here it must equal an independent pure-Python statement of
the same sums (zero padding written out by hand, the kernel reversed, Python
integers reduced modulo 2^bits) on small random 1-D and 2-D cases whose
products overflow every type, and reproduce the crate's u8 padding literal
(test_type_cast_safety, src/padding/mod.rs:619-624) through a one-tap
convolution.  No device work.
"""
import itertools

import numpy as np
import pytest

from helpers import ConvMode, PaddingMode, problem
from oracle import oracle as O

TYPES = [(O.DT_U8, np.uint8), (O.DT_I8, np.int8), (O.DT_I16, np.int16), (O.DT_U16, np.uint16),
         (O.DT_I32, np.int32), (O.DT_U32, np.uint32), (O.DT_I64, np.int64), (O.DT_U64, np.uint64)]


def _wrap(v, npt):
    bits = np.dtype(npt).itemsize * 8
    v %= 1 << bits
    if np.issubdtype(npt, np.signedinteger) and v >= 1 << (bits - 1):
        v -= 1 << bits
    return v


def _full_conv(x, k, npt):
    """Full-mode convolution with zero padding, as Python integers."""
    xs, ks = x.shape, k.shape
    pad = [kk - 1 for kk in ks]
    out_shape = [xs[i] + ks[i] - 1 for i in range(x.ndim)]
    y = np.zeros(out_shape, dtype=object)
    kr = k[tuple(slice(None, None, -1) for _ in ks)]  # convolution: reversed kernel
    for o in itertools.product(*[range(n) for n in out_shape]):
        acc = 0
        for t in itertools.product(*[range(n) for n in ks]):
            src = [o[i] + t[i] - pad[i] for i in range(x.ndim)]
            if all(0 <= src[i] < xs[i] for i in range(x.ndim)):
                acc += int(x[tuple(src)]) * int(kr[t])
        y[o] = _wrap(acc, npt)
    return y


@pytest.mark.parametrize("code,npt", TYPES)
def test_oracle_integer_sums_wrap_like_release_rust(code, npt):
    rng = np.random.default_rng(code)
    info = np.iinfo(npt)
    # large magnitudes so products overflow; 64-bit values stay exact in the
    # oracle's double-valued padding (|v| <= 2^53)
    hi = min(int(info.max), 1 << 40)
    lo = max(int(info.min), -(1 << 40))
    for shape, kshape in (((9,), (4,)), ((5, 6), (3, 2))):
        x = rng.integers(lo, hi, shape, dtype=np.int64, endpoint=True).astype(npt)
        k = rng.integers(lo, hi, kshape, dtype=np.int64, endpoint=True).astype(npt)
        st, y = O.conv(problem(code, x, k, ConvMode.Full, PaddingMode.Zeros), x, k)
        assert st == 0
        want = _full_conv(x, k, npt)
        assert y.dtype == npt
        assert [int(v) for v in y.ravel()] == [int(v) for v in want.ravel()], (npt, shape)


def test_u8_circular_padding_literal():
    """src/padding/mod.rs:619-624: [1u8, 2, 3] padded by one sample each side
    with Circular gives [3, 1, 2, 3, 1]; a one-tap kernel of 1 returns the
    padded array."""
    x = np.array([1, 2, 3], np.uint8)
    k = np.array([1], np.uint8)
    mode = ConvMode.Explicit([[1, 1]], [1])
    st, y = O.conv(problem(O.DT_U8, x, k, mode, PaddingMode.Circular), x, k)
    assert st == 0
    assert y.tolist() == [3, 1, 2, 3, 1]
