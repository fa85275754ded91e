"""The closed-form border map against the crate's sequential padding.

The crate materialises the padded array by filling axis 0, 1, 2 in order,
front then back, each cell copying a whole hyperplane out of the buffer's
current contents (src/padding/mod.rs:84-452, src/padding/dim.rs,
src/padding/half_dim.rs:30-343).  The library never stores that array: every
kernel evaluates a closed form of it (axis_map per axis, then the first
constant from the last axis, else pre-fill zero, else the input sample).
ndconv_padded_host evaluates the same closed form on the host; here it must
equal the oracle's literal sequential restatement exactly, on random N-d
cases with axes of 1-8 samples and pads up to 130 per side (the uneven
batch's tiny-axis, large-pad regime: reflect fronts reading unfilled back
pads, non-periodic circular fronts), every border kind on either side and
constant values; where the crate panics both report PadOutOfRange.  No
device work.
"""
import ctypes

import numpy as np
import pytest

from helpers import C64, F64, BorderType, ConvMode, PaddingMode, problem
from ndconv import _abi
from oracle import oracle as O


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()


def _border(rng):
    kind = int(rng.integers(0, 5))
    if kind == 1:
        return BorderType.Const(float(rng.integers(-9, 10)) + 0.5)
    return [BorderType.Zeros, None, BorderType.Reflect, BorderType.Replicate, BorderType.Circular][kind]


def _case(rng, max_pad):
    rank = int(rng.integers(1, 4))
    shape = [int(rng.integers(1, 9)) for _ in range(rank)]
    pads = [[int(rng.integers(0, max_pad + 1)) for _ in range(2)] for _ in range(rank)]
    # keep the padded volume small enough for a quick sweep
    while np.prod([n + p[0] + p[1] for n, p in zip(shape, pads)]) > 60000:
        a = int(np.argmax([p[0] + p[1] for p in pads]))
        pads[a] = [p // 2 for p in pads[a]]
    mode = ConvMode.Explicit(pads, [1] * rank)
    pick = int(rng.integers(0, 3))
    if pick == 0:
        pm = PaddingMode.Explicit([[_border(rng), _border(rng)] for _ in range(rank)])
    elif pick == 1:
        pm = PaddingMode.Custom([_border(rng) for _ in range(rank)])
    else:
        pm = [PaddingMode.Zeros, PaddingMode.Const(2.25), PaddingMode.Reflect, PaddingMode.Replicate,
              PaddingMode.Circular][int(rng.integers(0, 5))]
    return shape, mode, pm


def _library_padded(p, x):
    cplx = np.iscomplexobj(x)
    nc = 2 if cplx else 1
    xd = np.ascontiguousarray(x, dtype=np.complex128 if cplx else np.float64)
    # padded extents: the pads ConvMode::unfold gives this problem
    pd, _ = O.unfold(p)
    L = [x.shape[i] + pd[i][0] + pd[i][1] for i in range(x.ndim)]
    out = np.zeros(L, dtype=xd.dtype)
    st = _abi.lib().ndconv_padded_host(ctypes.byref(p), xd.ctypes.data, nc, out.ctypes.data)
    return st, out


@pytest.mark.parametrize("seed,max_pad,cplx", [(1, 6, False), (2, 40, False), (3, 130, False), (4, 130, True)])
def test_border_map_equals_sequential_padding(seed, max_pad, cplx):
    rng = np.random.default_rng(seed)
    n_ok = n_err = 0
    for _ in range(700):
        shape, mode, pm = _case(rng, max_pad)
        x = rng.standard_normal(shape)
        if cplx:
            x = x + 1j * rng.standard_normal(shape)
        k = np.ones([1] * len(shape))
        p = problem(C64 if cplx else F64, x, k, mode, pm)
        st_o, y_o = O.padding(p, x)
        st_l, y_l = _library_padded(p, x)
        assert (st_o == 0) == (st_l == 0), (shape, mode, pm, st_o, st_l)
        if st_o:
            assert st_l == _abi.ERR_PAD_OUT_OF_RANGE, (shape, mode, pm, st_l)
            n_err += 1
            continue
        assert y_l.shape == y_o.shape
        assert np.array_equal(y_l, y_o), (shape, mode, pm)
        n_ok += 1
    assert n_ok > 400
    if max_pad >= 40:
        assert n_err > 0  # the panicking reflect cases are part of the sweep
