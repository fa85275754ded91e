"""Row blocking of the sliding-window direct kernel.

A warp line holds RY output rows TY apart; when TY s1 is a multiple of d1
their input rows coincide, so one staged window feeds RY kernel rows.  Each
output still sums its taps in one order (kz, ky, residue, kx) whatever the
plan, so every (row sets TY, rows per line RY) plan must give bit-identical
results: i32 equal to the oracle (src/conv/mod.rs:170-197 with wrapping
arithmetic), f32 / c32 within 1e-5 normwise and f64 within 1e-9 of the f64
oracle, and the batch entry point equal to one call per instance.  With
every border constant zero the library may permute the axes; that choice
ignores the knobs, so it cannot change the summation order either.  Shapes
keep the axis-folding form from taking these problems (two axes above 256
samples, a non-zero constant border, or folded GEMMs far larger than the
direct sums).
"""
import numpy as np
import pytest

import ndconv
from ndconv import _abi
from ndconv.tiletune import tuning
from helpers import C32, C64, F64, I32, BorderType, ConvMode, PaddingMode, normwise_err, problem, with_dilation
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = [
    # shape, kernel, dilation, stride, padding
    ((300, 700), (11, 31), (2, 2), (1, 1), PaddingMode.Reflect),  # rows coincide from TY = 2
    ((257, 300), (7, 5), (1, 1), (1, 1), PaddingMode.Const(0.5)),  # d1 = 1: any TY
    ((290, 400), (5, 9), (3, 1), (1, 1), PaddingMode.Circular),  # d1 = 3: TY = 3, 6
    ((260, 520), (6, 7), (2, 1), (2, 1), PaddingMode.Replicate),  # s1 = d1 = 2
    ((280, 600), (4, 10), (2, 3), (1, 2), PaddingMode.Custom([BorderType.Const(1.5), BorderType.Reflect])),
    ((3, 40, 300), (3, 5, 7), (1, 2, 1), (1, 1, 1), PaddingMode.Const(0.25)),
    ((9, 1200), (3, 17), (1, 1), (1, 1), PaddingMode.Reflect),  # few rows: RY limited by the rows
    ((10, 100, 200), (5, 11, 31), (1, 1, 1), (1, 1, 1), PaddingMode.Zeros),  # axes may be permuted
]
PLANS = [{}] + [{_abi.TUNE_SW_TY: t, _abi.TUNE_SW_RY: r} for t in (1, 2, 4, 8) for r in (1, 2, 4)]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()


def _mode(kshape, dil, stride):
    keff = [k * d - d + 1 for k, d in zip(kshape, dil)]
    return ConvMode.Explicit([[(e - 1) // 2, e // 2] for e in keff], list(stride))


def _all_plans(x, kw, mode, pm):
    outs = []
    for knobs in PLANS:
        with tuning(knobs):
            outs.append(ndconv.conv(x, kw, mode, pm))
    return outs


@pytest.mark.parametrize("case", range(len(CASES)))
def test_plans_bit_identical_and_exact_i32(case):
    shape, kshape, dil, stride, pm = CASES[case]
    rng = np.random.default_rng(500 + case)
    mode = _mode(kshape, dil, stride)
    xi = rng.integers(-60, 60, shape).astype(np.int32)
    ki = rng.integers(-7, 8, kshape).astype(np.int32)
    ki.flat[5::11] = 0  # some zero taps: the branchy path of their kernel rows
    # integral constants for the integer copy
    if pm.kind == _abi.PAD_CONST:
        pm = PaddingMode.Const(2)
    elif pm.kind == _abi.PAD_CUSTOM:
        pm = PaddingMode.Custom([BorderType.Const(3), BorderType.Reflect])
    kw = with_dilation(ki, list(dil))
    st, yo = O.conv(problem(I32, xi, kw, mode, pm), xi, ki)
    assert st == 0
    for knobs, y in zip(PLANS, _all_plans(xi, kw, mode, pm)):
        assert np.array_equal(y, yo), knobs


@pytest.mark.parametrize("case", range(len(CASES)))
def test_plans_bit_identical_f32(case):
    shape, kshape, dil, stride, pm = CASES[case]
    rng = np.random.default_rng(600 + case)
    mode = _mode(kshape, dil, stride)
    x = rng.standard_normal(shape).astype(np.float32)
    k = rng.standard_normal(kshape).astype(np.float32)
    kw = with_dilation(k, list(dil))
    outs = _all_plans(x, kw, mode, pm)
    for knobs, y in zip(PLANS, outs):
        assert np.array_equal(y, outs[0]), knobs
    st, y64 = O.conv(problem(F64, x.astype(np.float64), with_dilation(k.astype(np.float64), list(dil)), mode, pm),
                     x.astype(np.float64), k.astype(np.float64))
    assert st == 0
    assert normwise_err(outs[0], y64) <= 1e-5


@pytest.mark.parametrize("dt", [F64, C32])
def test_plans_two_rows_per_line(dt):
    """f64 and c32 lines hold at most two rows."""
    shape, kshape, dil, stride, pm = CASES[0]
    rng = np.random.default_rng(700 + dt)
    mode = _mode(kshape, dil, stride)
    if dt == C32:
        x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
        k = (rng.standard_normal(kshape) + 1j * rng.standard_normal(kshape)).astype(np.complex64)
        x64, k64, d64, tol = x.astype(np.complex128), k.astype(np.complex128), C64, 1e-5
    else:
        x = rng.standard_normal(shape)
        k = rng.standard_normal(kshape)
        x64, k64, d64, tol = x, k, F64, 1e-9
    kw = with_dilation(k, list(dil))
    outs = _all_plans(x, kw, mode, pm)
    for knobs, y in zip(PLANS, outs):
        assert np.array_equal(y, outs[0]), knobs
    st, y64 = O.conv(problem(d64, x64, with_dilation(k64, list(dil)), mode, pm), x64, k64)
    assert st == 0
    assert normwise_err(outs[0], y64) <= tol


def test_batch_entry_matches_single_calls():
    """The batch entry point plans for many instances (more rows per line);
    its results equal one call per instance."""
    import torch
    shape, kshape, dil, stride, pm = CASES[0]
    mode = _mode(kshape, dil, stride)
    g = torch.Generator(device="cuda").manual_seed(5)
    xs = [torch.randn(shape, generator=g, device="cuda") for _ in range(12)]
    ks = [torch.randn(kshape, generator=g, device="cuda") for _ in range(12)]
    kws = [with_dilation(k, list(dil)) for k in ks]
    ys = ndconv.conv_batch(xs, kws, mode, pm)
    for i in range(12):
        assert torch.equal(ys[i], ndconv.conv(xs[i], kws[i], mode, pm)), i
