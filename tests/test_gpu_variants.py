"""GPU parity of every algorithm variant (the autotuner's candidates) and of
the sliding-window direct kernel at strides other than 1.

Every variant must meet the same bar as the default path: f32 / c32
normwise error <= 1e-5 against the f64 oracle, f64 <= 1e-9, i32 bit-exact.
"""
import numpy as np
import pytest

import ndconv
from ndconv import _abi
from helpers import (C32, C64, F32, F64, I32, BorderType, ConvMode, PaddingMode, normwise_err, problem,
                     with_dilation)
from oracle import oracle as O
from test_gpu_parity import _c2, _c3, _kw, _oracle64, random_case

pytestmark = pytest.mark.gpu
TOL32 = 1e-5
FFT_VARIANTS = [_abi.ALGO_FFT_ND, _abi.ALGO_FFT_RS, _abi.ALGO_FFT_ND_POW2, _abi.ALGO_FFT_RS_POW2]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()


@pytest.mark.parametrize("variant", FFT_VARIANTS)
@pytest.mark.parametrize("cfg", ["c2", "c3", "c3_complex"])
def test_fft_variants_full_size(variant, cfg):
    x, kw, mode, pm = {"c2": _c2, "c3": _c3, "c3_complex": lambda: _c3(True)}[cfg]()
    y64 = _oracle64(x, kw, mode, pm)
    y = ndconv.conv_algo(x, kw, mode, pm, variant)
    assert normwise_err(y, y64) <= TOL32


@pytest.mark.parametrize("variant", FFT_VARIANTS)
@pytest.mark.parametrize("rank", [1, 2, 3])
@pytest.mark.parametrize("dt", [F32, C32, F64])
def test_fft_variants_random(variant, rank, dt):
    rng = np.random.default_rng(7000 + 100 * variant + 10 * rank + dt)
    n_ok = 0
    for _ in range(25):
        shape, kshape, kw, mode, pmode = random_case(rng, rank)
        if dt == C32:
            x = (rng.random(shape) + 1j * rng.random(shape)).astype(np.complex64)
            k = (rng.random(kshape) + 1j * rng.random(kshape)).astype(np.complex64)
            dt64, ty = C64, np.complex128
        else:
            x = rng.random(shape).astype(np.float32 if dt == F32 else np.float64)
            k = rng.random(kshape).astype(x.dtype)
            dt64, ty = F64, np.float64
        st, y64 = O.conv(problem(dt64, x, _kw(kw, k), mode, pmode), x.astype(ty), k.astype(ty))
        if st:
            with pytest.raises(ndconv.ConvError):
                ndconv.conv_algo(x, _kw(kw, k), mode, pmode, variant)
            continue
        y = ndconv.conv_algo(x, _kw(kw, k), mode, pmode, variant)
        assert y.shape == y64.shape
        tol = TOL32 if dt != F64 else 1e-9
        assert normwise_err(y, y64) <= tol, (shape, kshape, mode, pmode, normwise_err(y, y64))
        n_ok += 1
    assert n_ok > 8


def test_fft_variant_rejects_i32():
    x = np.ones((8, 8), np.int32)
    with pytest.raises(ndconv.ConvError):
        ndconv.conv_algo(x, np.ones((3, 3), np.int32), ConvMode.Same, PaddingMode.Zeros, _abi.ALGO_FFT_RS)


# ---- sliding-window direct kernel at x-strides > 1 (residue classes x phases) ---------------
@pytest.mark.parametrize("shape,kshape,dil,stride,pm", [
    ((3, 700), (5, 9), (1, 2), (1, 2), PaddingMode.Reflect),         # gcd 2: one residue, one phase
    ((4, 901), (3, 11), (2, 1), (1, 2), PaddingMode.Circular),       # two residues
    ((2, 5, 640), (3, 3, 13), (1, 1, 2), (1, 2, 3), PaddingMode.Replicate),  # 3 residues x 2 phases
    ((5, 777), (7, 8), (1, 3), (2, 2), PaddingMode.Zeros),           # 2 residues x 3 phases
    ((2, 1000), (3, 21), (1, 3), (1, 3), PaddingMode.Const(2)),      # gcd 3
    ((6, 333), (4, 6), (2, 4), (3, 4), PaddingMode.Reflect),         # gcd 4
    ((2000,), (101,), 2, 2, PaddingMode.Replicate),
    ((2, 3000), (9, 51), 2, 2, PaddingMode.Circular),
])
def test_strided_sliding_window(shape, kshape, dil, stride, pm):
    rng = np.random.default_rng(sum(shape) + sum(kshape))
    r = len(shape)
    dil = list(dil) if isinstance(dil, tuple) else [dil] * r
    stride = list(stride) if isinstance(stride, tuple) else [stride] * r
    keff = [kshape[i] * dil[i] - dil[i] + 1 for i in range(r)]
    mode = ConvMode.Explicit([[(e - 1) // 2, e // 2] for e in keff], stride)
    xi = rng.integers(-50, 50, shape).astype(np.int32)
    ki = rng.integers(-5, 6, kshape).astype(np.int32)
    st, yo = O.conv(problem(I32, xi, with_dilation(ki, dil), mode, pm), xi, ki)
    assert st == 0
    assert np.array_equal(ndconv.conv(xi, with_dilation(ki, dil), mode, pm), yo)
    xf, kf = xi.astype(np.float32) / 7, ki.astype(np.float32) / 3
    y64 = _oracle64(xf, with_dilation(kf, dil), mode, pm)
    assert normwise_err(ndconv.conv(xf, with_dilation(kf, dil), mode, pm), y64) <= TOL32
    # zero taps inside the kernel take the branchy path; results stay exact
    ki2 = ki.copy()
    ki2.flat[::3] = 0
    st, yo2 = O.conv(problem(I32, xi, with_dilation(ki2, dil), mode, pm), xi, ki2)
    assert np.array_equal(ndconv.conv(xi, with_dilation(ki2, dil), mode, pm), yo2)


def test_batch_plan_fft_variants():
    import torch
    from ndconv.batch import BatchPlan
    from ndconv import workloads as W
    specs = W.uneven_batch(40, seed=11, max_log2=14, kmax=31)
    xs, ks = W.make_tensors(specs, seed=11)
    kws = [with_dilation(k, s.dilation) for k, s in zip(ks, specs)]
    modes = [(s.conv_mode(), s.padding_mode()) for s in specs]
    algos = [FFT_VARIANTS[i % 4] for i in range(len(specs))]
    plan = BatchPlan(modes, xs, kws, algos=algos)
    refs = [ndconv.conv_algo(xs[i], kws[i], *modes[i], algos[i]) for i in range(len(specs))]
    for graph in (False, True):
        for y in plan.outs:
            y.fill_(float("nan"))
        plan.run(graph=graph)
        plan.check()
        torch.cuda.synchronize()
        for i in range(len(specs)):
            assert torch.equal(plan.outs[i], refs[i]), (graph, i, specs[i], algos[i])
    plan.close()
