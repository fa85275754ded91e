"""GPU parity: the CUDA library (through the C ABI) against the oracle.

Bars: i32 direct conv bit-exact; f32 / c32 normwise error <= 1e-5 against
the f64 oracle (the stated tolerance); f64 / c64 <= 1e-12.
"""
import json
import os

import numpy as np
import pytest

import ndconv
from helpers import (C32, C64, F32, F64, I32, BorderType, ConvMode, PaddingMode, mode_from_json,
                     normwise_err, problem, with_dilation)
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "torch_cases.json")
TOL32 = 1e-5
TOL64 = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()
    yield


def test_library_loads_and_reports_version():
    assert b"sm_103a" in ndconv._abi.lib().ndconv_version()


# ---- padding literals re-asserted through conv with a 1-tap kernel ---------------------
from test_oracle_golden import PAD_CASES  # noqa: E402


@pytest.mark.parametrize("arr,pmode,pads,expected", PAD_CASES)
@pytest.mark.parametrize("algo", ["direct", "fft"])
def test_padding_literals_gpu(arr, pmode, pads, expected, algo):
    x = np.array(arr, dtype=np.float64 if algo == "fft" else np.int32)
    k = np.ones([1] * x.ndim, dtype=x.dtype)
    mode = ConvMode.Explicit(pads, [1] * x.ndim)
    f = ndconv.conv if algo == "direct" else ndconv.conv_fft
    y = f(x, k, mode, pmode)
    assert np.round(np.real(y)).astype(np.int64).tolist() == expected


def test_conv_vs_torch_fixture_gpu():
    doc = json.load(open(GOLD))
    for c in doc["conv"]:
        x = np.array(c["arr"], dtype=np.int32)
        k = np.array(c["kernel"], dtype=np.int32)
        kw = with_dilation(k, c["dilation"])
        if not c["reverse"]:
            kw = kw.no_reverse()
        y = ndconv.conv(x, kw, mode_from_json(c["mode"]), PaddingMode.Zeros)
        assert y.tolist() == c["expected"], c["name"]
        yf = ndconv.conv_fft(x.astype(np.float64), with_dilation(k.astype(np.float64), c["dilation"])
                             if c["reverse"] else with_dilation(k.astype(np.float64), c["dilation"]).no_reverse(),
                             mode_from_json(c["mode"]), PaddingMode.Zeros)
        assert np.round(yf).astype(np.int64).tolist() == c["expected"], c["name"]


@pytest.mark.parametrize("x,k,expected", [
    ([42], [2], [84]), ([1, 2, 3, 4], [3], [3, 6, 9, 12]), ([[1, 2], [3, 4]], [[1]], [[1, 2], [3, 4]]),
])
def test_conv_edge_literals_gpu(x, k, expected):
    x, k = np.array(x, dtype=np.int32), np.array(k, dtype=np.int32)
    assert ndconv.conv(x, k, ConvMode.Same, PaddingMode.Zeros).tolist() == expected
    yf = ndconv.conv_fft(x.astype(np.float32), k.astype(np.float32), ConvMode.Same, PaddingMode.Zeros)
    assert np.round(yf).astype(np.int64).tolist() == expected


def test_errors_gpu():
    x = np.ones((3, 3), dtype=np.float32)
    with pytest.raises(ndconv.DataShape):
        ndconv.conv(np.ones((0, 3), np.float32), np.ones((2, 2), np.float32), ConvMode.Same, PaddingMode.Zeros)
    with pytest.raises(ndconv.KernelShape):
        ndconv.conv(x, np.ones((0, 2), np.float32), ConvMode.Same, PaddingMode.Zeros)
    with pytest.raises(ndconv.DataShape):  # FFT path reports DataShape for the kernel
        ndconv.conv_fft(x, np.ones((0, 2), np.float32), ConvMode.Same, PaddingMode.Zeros)
    with pytest.raises(ndconv.MismatchShape):
        ndconv.conv(x, np.ones((5, 5), np.float32), ConvMode.Valid, PaddingMode.Zeros)
    with pytest.raises(ndconv.MismatchShape):
        ndconv.conv_fft(x, np.ones((5, 5), np.float32), ConvMode.Valid, PaddingMode.Zeros)
    # reflect panics upstream -> PaddingOutOfRange
    with pytest.raises(ndconv.PaddingOutOfRange):
        ndconv.conv(np.ones(2, np.float32), np.ones(1, np.float32), ConvMode.Explicit([[3, 0]], [1]),
                    PaddingMode.Reflect)
    # direct pads before the size check, FFT checks sizes first
    bad = (np.ones(2, np.float32), np.ones(9, np.float32), ConvMode.Explicit([[3, 0]], [1]), PaddingMode.Reflect)
    with pytest.raises(ndconv.PaddingOutOfRange):
        ndconv.conv(*bad)
    with pytest.raises(ndconv.MismatchShape):
        ndconv.conv_fft(*bad)
    with pytest.raises(ndconv.Unsupported):
        ndconv.conv_fft(np.ones(4, np.int32), np.ones(2, np.int32), ConvMode.Same, PaddingMode.Zeros)


# ---- randomized parity over the whole API surface --------------------------------------
BORDERS = [BorderType.Zeros, BorderType.Const(3.5), BorderType.Reflect, BorderType.Replicate,
           BorderType.Circular]


def random_case(rng, rank, max_n=24, max_k=7):
    shape = [int(rng.integers(1, max_n)) for _ in range(rank)]
    kshape = [int(rng.integers(1, max_k)) for _ in range(rank)]
    dil = [int(rng.integers(1, 4)) for _ in range(rank)]
    keff = [kshape[i] * dil[i] - dil[i] + 1 for i in range(rank)]
    m = rng.integers(0, 5)
    if m == 0:
        mode = ConvMode.Full
    elif m == 1:
        mode = ConvMode.Same
    elif m == 2:
        mode = ConvMode.Valid
        shape = [max(shape[i], keff[i]) for i in range(rank)]
    elif m == 3:
        pads = [int(rng.integers(0, keff[i] + 3)) for i in range(rank)]
        mode = ConvMode.Custom(pads, [int(rng.integers(1, 4)) for _ in range(rank)])
    else:
        pads = [[int(rng.integers(0, keff[i] + 3)), int(rng.integers(0, keff[i] + 3))] for i in range(rank)]
        mode = ConvMode.Explicit(pads, [int(rng.integers(1, 4)) for _ in range(rank)])
    pm = int(rng.integers(0, 7))
    if pm == 0:
        pmode = PaddingMode.Zeros
    elif pm == 1:
        pmode = PaddingMode.Const(-1.25)
    elif pm == 2:
        pmode = PaddingMode.Reflect
    elif pm == 3:
        pmode = PaddingMode.Replicate
    elif pm == 4:
        pmode = PaddingMode.Circular
    elif pm == 5:
        pmode = PaddingMode.Custom([BORDERS[int(rng.integers(0, 5))] for _ in range(rank)])
    else:
        pmode = PaddingMode.Explicit([[BORDERS[int(rng.integers(0, 5))], BORDERS[int(rng.integers(0, 5))]]
                                      for _ in range(rank)])
    kw = with_dilation(np.zeros(kshape), dil)
    if rng.integers(0, 2):
        kw = kw.no_reverse()
    return shape, kshape, kw, mode, pmode


def _kw(kw, k):
    out = with_dilation(k, kw.dilation)
    return out if kw.reverse_flag else out.no_reverse()


@pytest.mark.parametrize("rank", [1, 2, 3])
def test_random_direct_i32_bitexact(rank):
    rng = np.random.default_rng(100 + rank)
    n_ok = 0
    for _ in range(60):
        shape, kshape, kw, mode, pmode = random_case(rng, rank)
        x = rng.integers(-100, 100, shape).astype(np.int32)
        k = rng.integers(-5, 5, kshape).astype(np.int32)
        if pmode.kind == 1:
            pmode = PaddingMode.Const(7)
        if pmode.kind in (5, 6):  # integer constants for the i32 path
            pmode.borders = [[BorderType.Const(2) if b.kind == 1 else b for b in bs] if isinstance(bs, list)
                             else (BorderType.Const(2) if bs.kind == 1 else bs) for bs in pmode.borders]
        p = problem(I32, x, _kw(kw, k), mode, pmode)
        st, yo = O.conv(p, x, k)
        if st:
            with pytest.raises(ndconv.ConvError):
                ndconv.conv(x, _kw(kw, k), mode, pmode)
            continue
        y = ndconv.conv(x, _kw(kw, k), mode, pmode)
        assert y.dtype == np.int32 and np.array_equal(y, yo), (shape, kshape, mode, pmode)
        n_ok += 1
    assert n_ok > 20


@pytest.mark.parametrize("rank", [1, 2, 3])
@pytest.mark.parametrize("dt", [F32, C32, F64])
@pytest.mark.parametrize("algo", ["direct", "fft"])
def test_random_float_parity(rank, dt, algo):
    rng = np.random.default_rng(1000 * rank + 10 * dt + (algo == "fft"))
    f = ndconv.conv if algo == "direct" else ndconv.conv_fft
    n_ok = 0
    for _ in range(40):
        shape, kshape, kw, mode, pmode = random_case(rng, rank)
        if dt in (C32, C64):
            x = (rng.random(shape) + 1j * rng.random(shape)).astype(np.complex64 if dt == C32 else np.complex128)
            k = (rng.random(kshape) + 1j * rng.random(kshape)).astype(x.dtype)
            dt64 = C64
        else:
            x = rng.random(shape).astype(np.float32 if dt == F32 else np.float64)
            k = rng.random(kshape).astype(x.dtype)
            dt64 = F64
        p64 = problem(dt64, x, _kw(kw, k), mode, pmode)
        st, y64 = O.conv(p64, x.astype(np.complex128 if dt64 == C64 else np.float64),
                         k.astype(np.complex128 if dt64 == C64 else np.float64))
        if st:
            with pytest.raises(ndconv.ConvError):
                f(x, _kw(kw, k), mode, pmode)
            continue
        y = f(x, _kw(kw, k), mode, pmode)
        assert y.shape == y64.shape
        tol = TOL32 if dt in (F32, C32) else TOL64 * (10 if algo == "fft" else 1) * 1e3
        assert normwise_err(y, y64) <= tol, (shape, kshape, mode, pmode, normwise_err(y, y64))
        n_ok += 1
    assert n_ok > 15


def test_strided_views():
    rng = np.random.default_rng(7)
    import torch
    xb = torch.from_numpy(rng.random((40, 60)).astype(np.float32)).cuda()
    kb = torch.from_numpy(rng.random((9, 12)).astype(np.float32)).cuda()
    x = xb[::2, 1::3]          # non-contiguous view
    k = kb.t()[::2, ::3]       # transposed + strided kernel
    mode, pm = ConvMode.Same, PaddingMode.Custom([BorderType.Reflect, BorderType.Circular])
    xn, kn = x.cpu().numpy(), k.cpu().numpy()
    _, y64 = O.conv(problem(F64, xn, kn, mode, pm), xn.astype(np.float64), kn.astype(np.float64))
    for f in (ndconv.conv, ndconv.conv_fft):
        y = f(x, k, mode, pm).cpu().numpy()
        assert normwise_err(y, y64) <= TOL32


# ---- processor ----------------------------------------------------------------------------
@pytest.mark.parametrize("shape", [(6,), (7,), (2, 4), (3, 3), (5, 12), (4, 8, 8), (3, 5, 7), (16, 16)])
@pytest.mark.parametrize("dt", ["float64", "complex128", "float32"])
def test_processor_vs_oracle(shape, dt):
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(shape)
    if dt == "complex128":
        x = x + 1j * rng.standard_normal(shape)
    x = x.astype(dt)
    proc = ndconv.get_fft_processor(getattr(__import__("torch"), dt))
    spec = proc.forward(x)
    code = {"float64": O.DT_F64, "complex128": O.DT_C64, "float32": O.DT_F32}[dt]
    ref, ol = O.fft_forward(O.DT_F64 if code != O.DT_C64 else O.DT_C64, x.astype(
        np.float64 if dt != "complex128" else np.complex128))
    assert spec.shape == ref.shape
    tol = 1e-5 if dt == "float32" else 1e-11
    assert normwise_err(spec, ref) < tol
    back = proc.backward(spec)
    assert back.shape == x.shape
    assert normwise_err(back, x) < tol


# ---- the three benchmark cases at full size ---------------------------------------------------
def _c1():
    rng = np.random.default_rng(1)
    x = rng.random(5000).astype(np.float32)
    k = rng.random(31).astype(np.float32)
    return x, k, ConvMode.Full, PaddingMode.Zeros


def _c2(dtype=np.float32):
    rng = np.random.default_rng(2)
    if dtype == np.int32:
        x = rng.integers(-100, 101, (200, 5000)).astype(np.int32)
        k = rng.integers(-100, 101, (11, 31)).astype(np.int32)
    else:
        x = rng.random((200, 5000)).astype(dtype)
        k = rng.random((11, 31)).astype(dtype)
    return x, with_dilation(k, 2), ConvMode.Same, PaddingMode.Custom([BorderType.Reflect, BorderType.Circular])


def _c3(cplx=False):
    rng = np.random.default_rng(3)
    if cplx:
        x = (rng.standard_normal((10, 100, 200)) + 1j * rng.standard_normal((10, 100, 200))).astype(np.complex64)
        k = (rng.standard_normal((5, 11, 31)) + 1j * rng.standard_normal((5, 11, 31))).astype(np.complex64)
    else:
        x = rng.random((10, 100, 200)).astype(np.float32)
        k = rng.random((5, 11, 31)).astype(np.float32)
    return x, k, ConvMode.Same, PaddingMode.Zeros


def _oracle64(x, kw, mode, pm):
    k = kw.kernel if hasattr(kw, "kernel") else kw
    cplx = np.iscomplexobj(x)
    dt = C64 if cplx else F64
    p = problem(dt, x, kw, mode, pm)
    ty = np.complex128 if cplx else np.float64
    st, y = O.conv(p, x.astype(ty), np.asarray(k).astype(ty))
    assert st == 0
    return y


@pytest.mark.parametrize("cfg", ["c1", "c2", "c3", "c3_complex"])
@pytest.mark.parametrize("algo", ["direct", "fft"])
def test_benchmark_cases(cfg, algo):
    x, kw, mode, pm = {"c1": _c1, "c2": _c2, "c3": _c3, "c3_complex": lambda: _c3(True)}[cfg]()
    y64 = _oracle64(x, kw, mode, pm)
    f = ndconv.conv if algo == "direct" else ndconv.conv_fft
    y = f(x, kw, mode, pm)
    err = normwise_err(y, y64)
    assert err <= TOL32, err


def test_c2_i32_bitexact():
    x, kw, mode, pm = _c2(np.int32)
    p = problem(I32, x, kw, mode, pm)
    st, yo = O.conv(p, x, kw.kernel)
    assert st == 0
    y = ndconv.conv(x, kw, mode, pm)
    assert np.array_equal(y, yo)


# ---- batched submissions equal per-instance calls -------------------------------------------
@pytest.mark.parametrize("algo", ["direct", "fft"])
@pytest.mark.parametrize("cfg", [
    ((64, 300), (5, 9), 2, ConvMode.Same, PaddingMode.Custom([BorderType.Reflect, BorderType.Circular]), "float32"),
    ((6, 30, 40), (3, 4, 5), 1, ConvMode.Full, PaddingMode.Replicate, "complex64"),
    ((5000,), (31,), 1, ConvMode.Full, PaddingMode.Zeros, "float32"),
    ((50, 60), (7, 7), 1, ConvMode.Custom([2, 3], [2, 3]), PaddingMode.Circular, "float64"),
])
def test_batch_equals_single(algo, cfg):
    import torch
    xs_, ks_, dil, mode, pm, dt = cfg
    tdt = getattr(torch, dt)
    g = torch.Generator(device="cuda").manual_seed(5)
    n = 7
    if tdt.is_complex:
        xs = [torch.randn(xs_, generator=g, device="cuda", dtype=tdt) for _ in range(n)]
        ks = [torch.randn(ks_, generator=g, device="cuda", dtype=tdt) for _ in range(n)]
    else:
        xs = [torch.rand(xs_, generator=g, device="cuda", dtype=tdt) for _ in range(n)]
        ks = [torch.rand(ks_, generator=g, device="cuda", dtype=tdt) for _ in range(n)]
    kws = [with_dilation(k, dil) for k in ks]
    fb = ndconv.conv_batch if algo == "direct" else ndconv.conv_fft_batch
    f1 = ndconv.conv if algo == "direct" else ndconv.conv_fft
    yb = fb(xs, kws, mode, pm)
    for i in range(n):
        y1 = f1(xs[i], kws[i], mode, pm)
        assert torch.equal(yb[i], y1), i
    # and one instance against the f64 oracle
    x0, k0 = xs[0].cpu().numpy(), ks[0].cpu().numpy()
    y64 = _oracle64(x0, with_dilation(k0, dil), mode, pm)
    assert normwise_err(yb[0].cpu().numpy(), y64) <= TOL32


def test_batch_i32_bitexact():
    import torch
    g = torch.Generator(device="cuda").manual_seed(9)
    xs = [torch.randint(-100, 101, (200, 500), generator=g, device="cuda", dtype=torch.int32) for _ in range(5)]
    ks = [torch.randint(-100, 101, (11, 31), generator=g, device="cuda", dtype=torch.int32) for _ in range(5)]
    mode, pm = ConvMode.Same, PaddingMode.Custom([BorderType.Reflect, BorderType.Circular])
    ys = ndconv.conv_batch(xs, [with_dilation(k, 2) for k in ks], mode, pm)
    for x, k, y in zip(xs, ks, ys):
        p = problem(I32, x.cpu().numpy(), with_dilation(k.cpu().numpy(), 2), mode, pm)
        st, yo = O.conv(p, x.cpu().numpy(), k.cpu().numpy())
        assert st == 0 and np.array_equal(y.cpu().numpy(), yo)


# ---- taps that only ever read padding zeros ----------------------------------------------------
@pytest.mark.parametrize("shape,kshape,dil,stride,pm", [
    ((1, 1, 300), (9, 7, 5), 1, 1, PaddingMode.Reflect),
    ((2, 3, 257), (15, 13, 11), 2, 1, PaddingMode.Zeros),
    ((3, 2, 100), (11, 9, 7), 1, 2, PaddingMode.Circular),
    ((1, 500), (31, 9), 2, 2, PaddingMode.Zeros),
    ((4, 64), (25, 3), 1, 1, PaddingMode.Replicate),
])
def test_dead_taps_exact(shape, kshape, dil, stride, pm):
    rng = np.random.default_rng(sum(shape))
    keff = [k * dil - dil + 1 for k in kshape]
    mode = ConvMode.Explicit([[(e - 1) // 2, (e - 1) // 2] for e in keff], [stride] * len(shape))
    xi = rng.integers(-50, 50, shape).astype(np.int32)
    ki = rng.integers(-5, 6, kshape).astype(np.int32)
    p = problem(I32, xi, with_dilation(ki, dil), mode, pm)
    st, yo = O.conv(p, xi, ki)
    assert st == 0
    assert np.array_equal(ndconv.conv(xi, with_dilation(ki, dil), mode, pm), yo)
    xf, kf = xi.astype(np.float32) / 7, ki.astype(np.float32) / 3
    y64 = _oracle64(xf, with_dilation(kf, dil), mode, pm)
    assert normwise_err(ndconv.conv(xf, with_dilation(kf, dil), mode, pm), y64) <= TOL32
    # a non-finite weight where only padding zeros are read: NaN everywhere, like the oracle
    for bad in (np.nan, np.inf):
        kb = kf.copy()
        kb.flat[0] = bad  # corner tap (reversed: pairs with the far padding)
        st, yb = O.conv(problem(F64, xf, with_dilation(kb, dil), mode, pm), xf.astype(np.float64),
                        kb.astype(np.float64))
        y = ndconv.conv(xf, with_dilation(kb, dil), mode, pm)
        assert np.array_equal(np.isnan(y), np.isnan(yb))
        assert np.allclose(y[~np.isnan(y)], yb[~np.isnan(yb)], rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("shape,kshape,dil,stride,pm", [
    ((50, 1, 7), (9, 5, 11), 2, 2, PaddingMode.Replicate),
    ((300, 7, 2), (7, 9, 5), 2, 2, PaddingMode.Replicate),
    ((400, 3), (5, 7), 1, 2, PaddingMode.Reflect),
    ((9, 200, 2), (3, 5, 3), 1, 1, PaddingMode.Circular),
])
def test_long_leading_axis(shape, kshape, dil, stride, pm):
    # tiny contiguous output axis, long leading one (axes permuted for tiling)
    rng = np.random.default_rng(len(shape) + shape[0])
    keff = [k * dil - dil + 1 for k in kshape]
    mode = ConvMode.Explicit([[(e - 1) // 2, (e - 1) // 2] for e in keff], [stride] * len(shape))
    xi = rng.integers(-50, 50, shape).astype(np.int32)
    ki = rng.integers(-5, 6, kshape).astype(np.int32)
    st, yo = O.conv(problem(I32, xi, with_dilation(ki, dil), mode, pm), xi, ki)
    assert st == 0
    assert np.array_equal(ndconv.conv(xi, with_dilation(ki, dil), mode, pm), yo)
    xf, kf = xi.astype(np.float32) / 7, ki.astype(np.float32) / 3
    y64 = _oracle64(xf, with_dilation(kf, dil), mode, pm)
    assert normwise_err(ndconv.conv(xf, with_dilation(kf, dil), mode, pm), y64) <= TOL32
