"""Pin the oracle against the reference's own known answers (CPU only).

Literal vectors are the reference's test expectations, cited per case;
torch-derived expectations come from tests/golden/torch_cases.json
(tests/golden/make_golden.py), which recomputes the reference's LibTorch
comparisons.  FFT cases follow src/conv_fft/tests.rs with its tolerances.
"""
import json
import os

import numpy as np
import pytest

from helpers import (C32, C64, F32, F64, I32, BorderType, ConvMode, PaddingMode, mode_from_json,
                     problem, with_dilation)
from ndconv import no_reverse
from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden", "torch_cases.json")


def pad(arr, pmode, pads, fft_style=False):
    x = np.array(arr)
    k = np.ones([1] * x.ndim)
    p = problem(F64, x, k, ConvMode.Explicit(pads, [1] * x.ndim), pmode)
    st, out = O.padding(p, x, fft_style=fft_style)
    assert st == 0
    return out.real.astype(np.int64) if np.iscomplexobj(out) else out.astype(np.int64)


# ---- padding literal vectors: src/padding/mod.rs:464-759 -------------------------------
PAD_CASES = [
    ([1, 2, 3], PaddingMode.Zeros, [[1, 1]], [0, 1, 2, 3, 0]),
    ([[1, 2], [3, 4]], PaddingMode.Zeros, [[1, 1], [1, 1]],
     [[0, 0, 0, 0], [0, 1, 2, 0], [0, 3, 4, 0], [0, 0, 0, 0]]),
    ([[[1, 2]], [[3, 4]]], PaddingMode.Zeros, [[1, 0], [0, 1], [1, 0]],
     [[[0, 0, 0], [0, 0, 0]], [[0, 1, 2], [0, 0, 0]], [[0, 3, 4], [0, 0, 0]]]),
    ([1, 2, 3], PaddingMode.Zeros, [[2, 1]], [0, 0, 1, 2, 3, 0]),
    ([1, 2, 3], PaddingMode.Const(7), [[1, 1]], [7, 1, 2, 3, 7]),
    ([[1, 2], [3, 4]], PaddingMode.Const(9), [[1, 1], [1, 1]],
     [[9, 9, 9, 9], [9, 1, 2, 9], [9, 3, 4, 9], [9, 9, 9, 9]]),
    ([1, 2, 3], PaddingMode.Replicate, [[1, 2]], [1, 1, 2, 3, 3, 3]),
    ([[1, 2], [3, 4]], PaddingMode.Replicate, [[1, 1], [1, 1]],
     [[1, 1, 2, 2], [1, 1, 2, 2], [3, 3, 4, 4], [3, 3, 4, 4]]),
    ([1, 2], PaddingMode.Replicate, [[3, 3]], [1, 1, 1, 1, 2, 2, 2, 2]),
    ([1, 2, 3, 4], PaddingMode.Reflect, [[2, 2]], [3, 2, 1, 2, 3, 4, 3, 2]),
    ([[1, 2, 3], [4, 5, 6]], PaddingMode.Reflect, [[1, 1], [1, 1]],
     [[5, 4, 5, 6, 5], [2, 1, 2, 3, 2], [5, 4, 5, 6, 5], [2, 1, 2, 3, 2]]),
    ([1, 2, 3, 4], PaddingMode.Circular, [[2, 2]], [3, 4, 1, 2, 3, 4, 1, 2]),
    ([[1, 2], [3, 4]], PaddingMode.Circular, [[1, 1], [1, 1]],
     [[4, 3, 4, 3], [2, 1, 2, 1], [4, 3, 4, 3], [2, 1, 2, 1]]),
    ([1, 2, 3], PaddingMode.Circular, [[1, 1]], [3, 1, 2, 3, 1]),
    ([[1, 2], [3, 4]], PaddingMode.Custom([BorderType.Replicate, BorderType.Circular]),
     [[2, 2], [2, 2]],
     [[1, 2, 1, 2, 1, 2]] * 3 + [[3, 4, 3, 4, 3, 4]] * 3),
    ([[1, 2], [3, 4]], PaddingMode.Custom([BorderType.Reflect, BorderType.Const(7)]),
     [[2, 2], [2, 2]],
     [[7, 7, 0, 0, 7, 7], [7, 7, 3, 4, 7, 7], [7, 7, 1, 2, 7, 7], [7, 7, 3, 4, 7, 7],
      [7, 7, 1, 2, 7, 7], [7, 7, 3, 4, 7, 7]]),
    ([1, 2, 3], PaddingMode.Explicit([[BorderType.Const(7), BorderType.Const(9)]]), [[1, 2]],
     [7, 1, 2, 3, 9, 9]),
    ([1, 2, 3], PaddingMode.Zeros, [[0, 0]], [1, 2, 3]),
    ([42], PaddingMode.Replicate, [[2, 2]], [42, 42, 42, 42, 42]),
]


@pytest.mark.parametrize("arr,pmode,pads,expected", PAD_CASES)
@pytest.mark.parametrize("fft_style", [False, True])
def test_padding_literals(arr, pmode, pads, expected, fft_style):
    # padding (direct path) and padding_in (FFT path) must give the same buffer
    assert pad(arr, pmode, pads, fft_style).tolist() == expected


def test_padding_large_array():
    # src/padding/mod.rs:696-735
    arr = np.fromfunction(lambda i, j: i + j, (100, 100))
    out = pad(arr, PaddingMode.Zeros, [[5, 5], [5, 5]])
    assert out.shape == (110, 110)
    assert (out[:5] == 0).all() and (out[105:] == 0).all()
    assert (out[5:105, :5] == 0).all() and (out[5:105, 105:] == 0).all()
    assert out[5, 5] == 0 and out[54, 54] == 98 and out[104, 104] == 198


def test_padding_vs_torch_fixture():
    doc = json.load(open(GOLD))
    modes = {"Zeros": PaddingMode.Zeros, "Const": PaddingMode.Const(7),
             "Replicate": PaddingMode.Replicate, "Reflect": PaddingMode.Reflect,
             "Circular": PaddingMode.Circular}
    for c in doc["padding"]:
        got = pad(c["arr"], modes[c["mode"]], c["pads"])
        assert got.tolist() == c["expected"], c["name"]


def test_padding_panics_become_errors():
    # reflect front with p0 >= n + p1 and back with p1 >= p0 + n panic upstream
    x = np.array([1.0, 2.0])
    p = problem(F64, x, np.ones(1), ConvMode.Explicit([[3, 0]], [1]), PaddingMode.Reflect)
    assert O.padding(p, x)[0] == 4
    p = problem(F64, x, np.ones(1), ConvMode.Explicit([[0, 2]], [1]), PaddingMode.Reflect)
    assert O.padding(p, x)[0] == 4
    # circular with pad > n reads unfilled cells, giving the pre-fill value
    x = np.array([1.0, 2.0])
    p = problem(F64, x, np.ones(1), ConvMode.Explicit([[3, 3]], [1]), PaddingMode.Circular)
    st, out = O.padding(p, x)
    assert st == 0 and out.tolist() == [0, 1, 2, 1, 2, 1, 2, 1]


# ---- gen_offset_list: src/dilation/mod.rs:277-404 --------------------------------------
@pytest.mark.parametrize("k,dil,rev,strides,expected", [
    ([1.0, 2.0, 3.0], 1, True, [1], [(0, 3.0), (1, 2.0), (2, 1.0)]),
    ([1.0, 2.0, 3.0], 2, True, [1], [(0, 3.0), (2, 2.0), (4, 1.0)]),
    ([1.0, 2.0, 3.0], 2, False, [1], [(0, 1.0), (2, 2.0), (4, 3.0)]),
    ([[1.0, 2.0], [3.0, 4.0]], 1, True, [10, 1], [(0, 4.0), (1, 3.0), (10, 2.0), (11, 1.0)]),
    ([[1.0, 2.0], [3.0, 4.0]], [2, 3], True, [10, 1], [(0, 4.0), (3, 3.0), (20, 2.0), (23, 1.0)]),
    ([42.0], 5, True, [1], [(0, 42.0)]),
    ([0.0, 0.0, 0.0], 2, True, [1], []),
])
def test_offset_list(k, dil, rev, strides, expected):
    k = np.array(k)
    kw = with_dilation(k, dil)
    if not rev:
        kw = kw.no_reverse()
    p = problem(F64, np.zeros(k.shape), kw, ConvMode.Valid, PaddingMode.Zeros)
    got = [(o, float(v)) for o, v in O.taps(p, k, strides)]
    assert got == expected


def test_offset_list_filters_zeros():
    k = np.array([1.0, 0.0, 2.0, 0.0, 3.0])
    p = problem(F64, np.zeros(5), k, ConvMode.Valid, PaddingMode.Zeros)
    assert len(O.taps(p, k, [1])) == 3


# ---- good_size: src/conv_fft/good_size.rs -------------------------------------------------
def test_good_size_values():
    # exact powers and the /4*3, /6*5 descent with integer floor
    assert [O.good_size(n) for n in (1, 2, 3, 4, 5, 7, 8, 9)] == [1, 2, 3, 4, 5, 8, 8, 9]
    assert O.good_size(5060) == 5120 and O.good_size(220) == 256
    assert O.good_size(14) == 16 and O.good_size(110) == 128 and O.good_size(230) == 256
    for n in range(1, 3000):
        g = O.good_size(n)
        assert g >= n


# ---- direct conv vs the torch-computed expectations ------------------------------------
def test_conv_vs_torch_fixture():
    doc = json.load(open(GOLD))
    for c in doc["conv"]:
        x = np.array(c["arr"], dtype=np.int32)
        k = np.array(c["kernel"], dtype=np.int32)
        kw = with_dilation(k, c["dilation"])
        if not c["reverse"]:
            kw = kw.no_reverse()
        p = problem(I32, x, kw, mode_from_json(c["mode"]), PaddingMode.Zeros)
        st, y = O.conv(p, x, k)
        assert st == 0, c["name"]
        assert y.tolist() == c["expected"], c["name"]
        # f64 and f32 instantiations agree exactly on these integer inputs
        for dt in (F32, F64):
            p.dtype = dt
            st, yf = O.conv(p, x, k)
            assert np.array_equal(yf, np.array(c["expected"])), c["name"]


# src/conv/tests.rs:552-584
@pytest.mark.parametrize("x,k,expected", [
    ([42], [2], [84]),
    ([1, 2, 3, 4], [3], [3, 6, 9, 12]),
    ([[1, 2], [3, 4]], [[1]], [[1, 2], [3, 4]]),
])
def test_conv_edge_literals(x, k, expected):
    x, k = np.array(x, dtype=np.int32), np.array(k, dtype=np.int32)
    st, y = O.conv(problem(I32, x, k, ConvMode.Same, PaddingMode.Zeros), x, k)
    assert st == 0 and y.tolist() == expected


def test_conv_error_codes():
    x = np.zeros((0, 3), dtype=np.int32)
    k = np.ones((2, 2), dtype=np.int32)
    assert O.conv(problem(I32, x, k, ConvMode.Same, PaddingMode.Zeros), x, k)[0] == 1
    x = np.ones((3, 3), dtype=np.int32)
    k0 = np.ones((0, 2), dtype=np.int32)
    assert O.conv(problem(I32, x, k0, ConvMode.Same, PaddingMode.Zeros), x, k0)[0] == 2
    # FFT path reports the zero-size kernel as DataShape (src/conv_fft/mod.rs:211-212)
    p = problem(F32, x, k0, ConvMode.Same, PaddingMode.Zeros)
    assert O.conv_fft(p, x, k0)[0] == 1
    k5 = np.ones((5, 5), dtype=np.int32)
    assert O.conv(problem(I32, x, k5, ConvMode.Valid, PaddingMode.Zeros), x, k5)[0] == 3
    assert O.conv_fft(problem(F32, x, k5, ConvMode.Valid, PaddingMode.Zeros), x, k5)[0] == 3


# ---- FFT buffers: src/conv_fft/padding.rs:123-181 -------------------------------------
def test_fft_data_buffer():
    x = np.array([[1, 2], [3, 4]])
    k = np.ones((3, 3))
    p = problem(F64, x, k, ConvMode.Full,
                PaddingMode.Custom([BorderType.Const(7), BorderType.Const(8)]))
    st, d, _ = O.fft_buffers(p, [8, 8], x, k)
    assert st == 0
    assert d.astype(int).tolist() == [
        [8, 8, 7, 7, 8, 8, 0, 0], [8, 8, 7, 7, 8, 8, 0, 0], [8, 8, 1, 2, 8, 8, 0, 0],
        [8, 8, 3, 4, 8, 8, 0, 0], [8, 8, 7, 7, 8, 8, 0, 0], [8, 8, 7, 7, 8, 8, 0, 0],
        [0] * 8, [0] * 8]


def test_fft_kernel_buffer():
    x = np.array([[1, 2], [3, 4]])
    k = np.array([[1, 2, 3], [4, 5, 6], [7, 8, 9]])
    p = problem(F64, x, with_dilation(k, [2, 3]), ConvMode.Full, PaddingMode.Zeros)
    st, _, kb = O.fft_buffers(p, [8, 8], x, k)
    assert st == 0
    assert kb.astype(int).tolist() == [
        [1, 0, 0, 2, 0, 0, 3, 0], [0] * 8, [4, 0, 0, 5, 0, 0, 6, 0], [0] * 8,
        [7, 0, 0, 8, 0, 0, 9, 0], [0] * 8, [0] * 8, [0] * 8]


# ---- oracle FFT against numpy (third-party DFT) -----------------------------------------
@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 8, 12, 15, 16, 30, 97, 128, 210, 257, 1000, 1009])
def test_oracle_fft1d_vs_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    np.testing.assert_allclose(O.fft1d(x), np.fft.fft(x), rtol=1e-10, atol=1e-10 * n)
    np.testing.assert_allclose(O.fft1d(x, inverse=True), np.fft.ifft(x) * n, rtol=1e-10,
                               atol=1e-10 * n)


@pytest.mark.parametrize("shape", [(6,), (5,), (2, 4), (3, 3), (3, 5), (4, 8, 8), (3, 5, 7), (2, 3, 4),
                                   # many rows: blocks of batched transforms and their remainders,
                                   # mixed radices 2/3/4/5/7, a Bluestein length (257)
                                   (37, 60), (21, 210), (3, 37, 30), (18, 257), (6, 35, 18)])
def test_processor_layout_vs_numpy(shape):
    """Processor::forward's rotated layout: 1-D as is, 2-D (k1, k0), 3-D (k1, k2, k0)."""
    rng = np.random.default_rng(len(shape))
    x = rng.standard_normal(shape)
    spec, ol = O.fft_forward(O.DT_F64, x)
    ref = np.fft.rfftn(x)
    perm = {1: (0,), 2: (1, 0), 3: (1, 2, 0)}[len(shape)]
    np.testing.assert_allclose(spec, np.transpose(ref, perm), rtol=1e-9, atol=1e-9)
    assert ol == shape[-1]
    back = O.fft_backward(O.DT_F64, spec, ol)
    np.testing.assert_allclose(back, x, atol=1e-10)  # round trip, real.rs:291-478
    xc = x + 1j * rng.standard_normal(shape)
    specc, _ = O.fft_forward(O.DT_C64, xc)
    np.testing.assert_allclose(specc, np.transpose(np.fft.fftn(xc), perm), rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(O.fft_backward(O.DT_C64, specc, 0), xc, atol=1e-10)


@pytest.mark.parametrize("shape", [(37, 60), (21, 210), (3, 37, 30), (6, 35, 18)])
def test_processor_layout_vs_numpy_f32(shape):
    """The single-precision instantiation of the same transforms (the one the
    timed CPU baseline runs), batched over many rows."""
    rng = np.random.default_rng(len(shape) + shape[-1])
    x = rng.standard_normal(shape)
    perm = {2: (1, 0), 3: (1, 2, 0)}[len(shape)]
    spec, ol = O.fft_forward(O.DT_F32, x.astype(np.float32))
    ref = np.transpose(np.fft.rfftn(x), perm)
    assert np.linalg.norm(spec - ref) / np.linalg.norm(ref) < 1e-6
    back = O.fft_backward(O.DT_F32, spec, ol)
    assert np.abs(back - x).max() < 1e-5
    xc = x + 1j * rng.standard_normal(shape)
    specc, _ = O.fft_forward(O.DT_C32, xc.astype(np.complex64))
    refc = np.transpose(np.fft.fftn(xc), perm)
    assert np.linalg.norm(specc - refc) / np.linalg.norm(refc) < 1e-6


def test_fft_conv_f32_many_rows_vs_direct():
    """conv_fft in f32 on a case with many rows (batched transforms) against
    the f64 direct loop, with every border kind on one axis or the other."""
    rng = np.random.default_rng(11)
    x = rng.random((64, 300))
    k = rng.random((7, 9))
    for pm in (PaddingMode.Zeros, PaddingMode.Reflect, PaddingMode.Circular, PaddingMode.Replicate,
               PaddingMode.Const(0.5)):
        kw = with_dilation(k, 2)
        st, y64 = O.conv(problem(F64, x, kw, ConvMode.Same, pm), x, k)
        assert st == 0
        for nth in (1, 4):
            st, y32 = O.conv_fft(problem(F32, x, kw, ConvMode.Same, pm), x.astype(np.float32),
                                 k.astype(np.float32), nth)
            assert st == 0
            assert np.linalg.norm(y32 - y64) / np.linalg.norm(y64) < 1e-5, (pm, nth)


# ---- FFT conv vs direct conv: src/conv_fft/tests.rs:151-618, 799-857 ----------------------
def fft_vs_direct(x, kw, mode, pmode, dt, tol):
    x = np.array(x)
    k = kw.kernel if hasattr(kw, "kernel") else np.array(kw)
    pi = problem(I32, x, kw, mode, pmode)
    st, yi = O.conv(pi, x.astype(np.int32), np.asarray(k).astype(np.int32))
    assert st == 0
    pf = problem(dt, x, kw, mode, pmode)
    st, yf = O.conv_fft(pf, x, k)
    assert st == 0
    assert yf.shape == yi.shape
    assert np.abs(np.round(yf) - yi).max() < tol


T32, T64 = 1e-5, 1e-9


def test_fft_vs_direct_cases():
    A = np.array
    fft_vs_direct([1, 2, 3, 4, 5, 6], with_dilation(A([1, 1, 1, 1]), 2), ConvMode.Same,
                  PaddingMode.Zeros, F32, T32)
    fft_vs_direct([1, 2, 3, 4, 5], A([1, 2, 1]), ConvMode.Full, PaddingMode.Zeros, F64, T64)
    fft_vs_direct([1, 2, 3, 4, 5, 6], A([1, 1, 1]), ConvMode.Valid, PaddingMode.Zeros, F32, T32)
    fft_vs_direct([[1, 2], [3, 4], [5, 6], [7, 8], [9, 10], [11, 12]], A([[1, 0], [3, 1]]),
                  ConvMode.Same, PaddingMode.Replicate, F64, T64)
    fft_vs_direct([[1, 2], [3, 4]], with_dilation(A([[1, 0], [3, 1]]), 2).no_reverse(),
                  ConvMode.Custom([3, 3], [2, 2]), PaddingMode.Replicate, F64, T64)
    fft_vs_direct([[1, 2], [3, 4]], A([[1, 1], [1, 1]]), ConvMode.Full, PaddingMode.Zeros, F32, T32)
    fft_vs_direct([[1, 2, 3], [4, 5, 6], [7, 8, 9]], A([[1, 1], [1, 1]]), ConvMode.Valid,
                  PaddingMode.Zeros, F64, T64)
    fft_vs_direct([[[1, 2], [3, 4]], [[5, 6], [7, 8]]], np.ones((2, 3, 3), int), ConvMode.Same,
                  PaddingMode.Zeros, F32, T32)
    fft_vs_direct([[[1, 2]], [[3, 4]]], np.ones((2, 1, 2), int), ConvMode.Full, PaddingMode.Zeros,
                  F64, T64)
    fft_vs_direct([[[1, 2, 3], [4, 5, 6]], [[7, 8, 9], [10, 11, 12]]], np.ones((2, 1, 2), int),
                  ConvMode.Valid, PaddingMode.Zeros, F32, T32)
    fft_vs_direct([[1, 2, 3], [4, 5, 6]], np.ones((2, 2), int), ConvMode.Same,
                  PaddingMode.Replicate, F32, T32)
    fft_vs_direct([[1, 2, 3], [4, 5, 6]], np.ones((2, 2), int), ConvMode.Same, PaddingMode.Zeros,
                  F64, T64)
    fft_vs_direct([[1, 2], [3, 4]], np.ones((2, 2), int), ConvMode.Full, PaddingMode.Const(7),
                  F32, T32)
    fft_vs_direct([42], A([2]), ConvMode.Same, PaddingMode.Zeros, F32, T32)
    big = np.fromfunction(lambda i, j: (i + j) % 10, (50, 50)).astype(int)
    fft_vs_direct(big, A([[1, 2, 1], [2, 4, 2], [1, 2, 1]]), ConvMode.Same, PaddingMode.Zeros,
                  F64, 1e-8)


def test_fft_circular_1d():
    # src/conv_fft/tests.rs:216-242, tolerance 1e-6
    x = np.array([0.0, 0.1, 0.3, 0.4] * 4, dtype=np.float32)
    k = np.array([0.1, 0.3, 0.6, 0.3, 0.1], dtype=np.float32)
    p = problem(F32, x, k, ConvMode.Same, PaddingMode.Circular)
    _, yd = O.conv(p, x, k)
    _, yf = O.conv_fft(p, x, k)
    assert np.abs(yd - yf).max() < 1e-6


def test_complex_fft_vs_direct():
    # the reference's complex cases (src/conv_fft/tests.rs:172-207,339-374,448-507) compare
    # conv_fft with itself; here the complex FFT path is checked against direct conv
    rng = np.random.default_rng(3)
    for shape, kshape, kw, mode, pm in [
        ((6,), (4,), 2, ConvMode.Same, PaddingMode.Zeros),
        ((2, 2), (2, 2), 2, ConvMode.Custom([3, 3], [2, 2]), PaddingMode.Replicate),
        ((2, 2, 2), (2, 3, 3), 1, ConvMode.Same, PaddingMode.Zeros),
        ((7, 9), (3, 4), 1, ConvMode.Full, PaddingMode.Custom([BorderType.Reflect, BorderType.Const(1 + 2j)])),
    ]:
        x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        k = rng.standard_normal(kshape) + 1j * rng.standard_normal(kshape)
        kk = with_dilation(k, kw)
        if isinstance(mode, ConvMode) and mode.kind == 3:
            kk = kk.no_reverse()
        p = problem(C64, x, kk, mode, pm)
        st, yd = O.conv(p, x, k)
        assert st == 0
        st, yf = O.conv_fft(p, x, k)
        assert st == 0
        np.testing.assert_allclose(yf, yd, atol=1e-9)


def test_fft_par_equals_serial():
    # src/conv_fft/tests.rs:626-795 (par vs serial, 1e-4 f32 / 1e-9 f64)
    arr = np.fromfunction(lambda i, j: (i + j) % 10, (32, 32)).astype(np.float32)
    ker = np.array([[1.0, 2, 1], [0, 0, 0], [-1, -2, -1]], dtype=np.float32)
    for mode in (ConvMode.Same, ConvMode.Valid, ConvMode.Full):
        p = problem(F32, arr, ker, mode, PaddingMode.Zeros)
        _, s = O.conv_fft(p, arr, ker, 1)
        _, q = O.conv_fft(p, arr, ker, 4)
        assert np.abs(s - q).max() < 1e-4
    a3 = np.fromfunction(lambda i, j, k: (i + j + k) % 5, (16, 16, 16)).astype(np.float64)
    k3 = -np.ones((3, 3, 3))
    k3[1, 1, 1] = 8
    p = problem(F64, a3, k3, ConvMode.Same, PaddingMode.Zeros)
    _, s = O.conv_fft(p, a3, k3, 1)
    _, q = O.conv_fft(p, a3, k3, 3)
    assert np.abs(s - q).max() < 1e-9


def test_no_reverse_is_correlation():
    rng = np.random.default_rng(0)
    x = rng.integers(-5, 5, (9, 11)).astype(np.int32)
    k = rng.integers(-3, 3, (3, 4)).astype(np.int32)
    _, a = O.conv(problem(I32, x, no_reverse(k), ConvMode.Valid, PaddingMode.Zeros), x, k)
    kf = np.ascontiguousarray(k[::-1, ::-1])
    _, b = O.conv(problem(I32, x, kf, ConvMode.Valid, PaddingMode.Zeros), x, kf)
    assert np.array_equal(a, b)
