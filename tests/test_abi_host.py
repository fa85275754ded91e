"""CPU checks of the C ABI: the library loads, exports every function that
include/ndconv.h declares, and its host-side planning (output shapes and
the reference's error order) agrees with the oracle.  No device calls."""
import ctypes
import os
import re

import numpy as np
import pytest

import ndconv
from helpers import F32, I32, ConvMode, PaddingMode, problem
from ndconv import _abi
from oracle import oracle as O
from test_gpu_parity import random_case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()


def declared_functions():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(ndconv_\w+)\s*\(", src, re.M)
    return sorted(set(names))


def test_exports_every_declared_symbol():
    L = ctypes.CDLL(_abi.LIB_PATH)
    names = declared_functions()
    assert "ndconv_conv" in names and "ndconv_conv_fft" in names
    for n in names:
        assert hasattr(L, n), n


def _abi_shape(p, algo):
    sh = (ctypes.c_int64 * 3)()
    st = _abi.lib().ndconv_output_shape(ctypes.byref(p), algo, sh)
    return st, [sh[i] for i in range(p.rank)]


@pytest.mark.parametrize("rank", [1, 2, 3])
def test_output_shape_and_errors_match_oracle(rank):
    rng = np.random.default_rng(rank)
    for _ in range(300):
        shape, kshape, kw, mode, pmode = random_case(rng, rank, max_n=6, max_k=5)
        if rng.integers(0, 10) == 0:
            shape[int(rng.integers(0, rank))] = 0
        if rng.integers(0, 10) == 0:
            kshape[int(rng.integers(0, rank))] = 0
        x = np.ones(shape, np.float32)
        k = np.ones(kshape, np.float32)
        kk = ndconv.with_dilation(k, kw.dilation)
        if not kw.reverse_flag:
            kk = kk.no_reverse()
        # direct path (i32 oracle), FFT path (f32 oracle)
        p = problem(I32, x, kk, mode, pmode)
        st_o, y = O.conv(p, x.astype(np.int32), k.astype(np.int32))
        st_a, sh = _abi_shape(p, 0)
        assert st_a == st_o, (shape, kshape, mode, pmode)
        if st_o == 0:
            assert sh == list(y.shape)
        p = problem(F32, x, kk, mode, pmode)
        st_o, y = O.conv_fft(p, x, k)
        st_a, sh = _abi_shape(p, 1)
        assert st_a == st_o, (shape, kshape, mode, pmode)
        if st_o == 0:
            assert sh == list(y.shape)


def test_last_error_message():
    x = np.ones((3, 3), np.float32)
    p = problem(F32, x, np.ones((5, 5), np.float32), ConvMode.Valid, PaddingMode.Zeros)
    st, _ = _abi_shape(p, 0)
    assert st == _abi.ERR_MISMATCH_SHAPE
    assert "ConvMode" in _abi.last_error()


def test_unsupported_ranks_and_element_types_are_refused():
    """The crate is generic over rank and element type; the library takes
    ranks 1..3, f32/f64/c32/c64 and the 8- to 64-bit integers, and refuses
    the rest (no fallback)."""
    from helpers import with_dilation
    p = problem(F32, np.ones((4, 5)), np.ones((3, 3)), ConvMode.Same, PaddingMode.Zeros)
    sh = (ctypes.c_int64 * 3)()
    q = _abi.Problem.from_buffer_copy(p)
    q.rank = 4
    assert _abi.lib().ndconv_output_shape(ctypes.byref(q), 0, sh) == _abi.ERR_UNSUPPORTED
    assert "rank" in _abi.last_error()
    for code in (12, 13, 100, -1):  # no such element type in the ABI
        q = _abi.Problem.from_buffer_copy(p)
        q.dtype = code
        assert _abi.lib().ndconv_output_shape(ctypes.byref(q), 0, sh) == _abi.ERR_UNSUPPORTED
        assert "element type" in _abi.last_error()
    q = _abi.Problem.from_buffer_copy(p)
    q.rank = 0
    assert _abi.lib().ndconv_output_shape(ctypes.byref(q), 0, sh) == _abi.ERR_INVALID
    for dt in (np.float16, np.bool_):
        with pytest.raises(ndconv.Unsupported):
            ndconv.api.dtype_code(np.dtype(dt))
    for dt, code in ((np.int8, _abi.I8), (np.uint8, _abi.U8), (np.int16, _abi.I16), (np.uint16, _abi.U16),
                     (np.uint32, _abi.U32), (np.int64, _abi.I64), (np.uint64, _abi.U64)):
        assert ndconv.api.dtype_code(np.dtype(dt)) == code
    with pytest.raises(ndconv.Unsupported):
        ndconv.build_problem(F32, (2, 2, 2, 2), with_dilation(np.ones((1, 1, 1, 1)), 1), ConvMode.Same,
                             PaddingMode.Zeros)
