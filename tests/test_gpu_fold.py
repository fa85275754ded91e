"""Axis folding (tiny axes with long kernels summed per input sample before
the convolution) against the oracle: i32 bit-exact, f32 / c32 within 1e-5,
the reference's NaN pattern for non-finite inputs, and batched == single."""
import numpy as np
import pytest

import ndconv
from helpers import C64, F64, I32, BorderType, ConvMode, PaddingMode, normwise_err, problem, with_dilation
from oracle import oracle as O
from test_gpu_parity import _oracle64

pytestmark = pytest.mark.gpu
TOL32 = 1e-5

CASES = [
    ((300, 6, 5), (9, 21, 17), 1, 1, PaddingMode.Replicate),
    ((200, 7, 3), (7, 15, 13), 2, 1, PaddingMode.Circular),
    ((150, 4, 9), (11, 13, 25), 2, 2, PaddingMode.Reflect),
    ((5, 300, 3), (13, 5, 31), 1, 2, PaddingMode.Zeros),
    ((4, 3, 500), (15, 17, 5), 2, 1, PaddingMode.Custom([BorderType.Circular, BorderType.Replicate,
                                                         BorderType.Reflect])),
    ((2, 900), (41, 7), 2, 1, PaddingMode.Replicate),
    # dilation above the folded extents: several taps per sample, empty buckets
    ((3, 2, 700), (17, 31, 9), 5, 2, PaddingMode.Circular),
    ((1, 4, 900), (9, 21, 5), 3, 1, PaddingMode.Replicate),
    ((2, 700, 3), (23, 5, 41), 4, 3, PaddingMode.Custom([BorderType.Reflect, BorderType.Circular,
                                                         BorderType.Replicate])),
]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()


def _mode(kshape, dil, stride):
    keff = [k * dil - dil + 1 for k in kshape]
    return ConvMode.Explicit([[(e - 1) // 2, (e - 1) // 2] for e in keff], [stride] * len(kshape))


@pytest.mark.parametrize("shape,kshape,dil,stride,pm", CASES)
def test_fold_i32_and_f32(shape, kshape, dil, stride, pm):
    rng = np.random.default_rng(sum(shape) + sum(kshape))
    mode = _mode(kshape, dil, stride)
    xi = rng.integers(-50, 50, shape).astype(np.int32)
    ki = rng.integers(-5, 6, kshape).astype(np.int32)
    st, yo = O.conv(problem(I32, xi, with_dilation(ki, dil), mode, pm), xi, ki)
    assert st == 0
    assert np.array_equal(ndconv.conv(xi, with_dilation(ki, dil), mode, pm), yo)
    xf, kf = (xi.astype(np.float32) / 7), (ki.astype(np.float32) / 3)
    y64 = _oracle64(xf, with_dilation(kf, dil), mode, pm)
    assert normwise_err(ndconv.conv(xf, with_dilation(kf, dil), mode, pm), y64) <= TOL32
    # no_reverse
    kwr = with_dilation(kf, dil).no_reverse()
    st, y64r = O.conv(problem(F64, xf, kwr, mode, pm), xf.astype(np.float64), kf.astype(np.float64))
    assert normwise_err(ndconv.conv(xf, kwr, mode, pm), y64r) <= TOL32


def test_fold_complex():
    rng = np.random.default_rng(4)
    shape, kshape = (120, 5, 4), (9, 15, 13)
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    k = (rng.standard_normal(kshape) + 1j * rng.standard_normal(kshape)).astype(np.complex64)
    mode, pm = _mode(kshape, 1, 1), PaddingMode.Replicate
    st, y64 = O.conv(problem(C64, x, k, mode, pm), x.astype(np.complex128), k.astype(np.complex128))
    assert normwise_err(ndconv.conv(x, k, mode, pm), y64) <= TOL32


@pytest.mark.parametrize("where", ["data", "kernel"])
def test_fold_nonfinite_follows_reference(where):
    rng = np.random.default_rng(5)
    shape, kshape = (100, 5, 4), (7, 15, 13)
    x = rng.random(shape).astype(np.float32)
    k = rng.random(kshape).astype(np.float32)
    if where == "data":
        x[40, 2, 1] = np.inf
    else:
        k[3, 0, 12] = np.nan
    mode, pm = _mode(kshape, 1, 1), PaddingMode.Reflect
    st, y64 = O.conv(problem(F64, x, k, mode, pm), x.astype(np.float64), k.astype(np.float64))
    y = ndconv.conv(x, k, mode, pm)
    assert np.array_equal(np.isnan(y), np.isnan(y64)) and np.array_equal(np.isinf(y), np.isinf(y64))
    fin = np.isfinite(y64)
    assert np.allclose(y[fin], y64[fin], rtol=1e-4, atol=1e-4)


def test_fold_in_batch_plan_equals_single():
    import torch
    from ndconv.batch import BatchPlan
    g = torch.Generator(device="cuda").manual_seed(3)
    shapes = [((300, 6, 5), (9, 21, 17)), ((200, 7, 3), (7, 15, 13)), ((64, 300), (5, 9)), ((5000,), (31,))]
    xs = [torch.rand(s, generator=g, device="cuda") for s, _ in shapes]
    ks = [torch.rand(k, generator=g, device="cuda") for _, k in shapes]
    kws = [with_dilation(k, 1) for k in ks]
    modes = [(_mode(k, 1, 1), PaddingMode.Replicate) for _, k in shapes]
    plan = BatchPlan(modes, xs, kws, algos=[0] * len(shapes))
    refs = [ndconv.conv(xs[i], kws[i], *modes[i]) for i in range(len(shapes))]
    for graph in (False, True):
        for y in plan.outs:
            y.fill_(float("nan"))
        plan.run(graph=graph)
        plan.check()
        torch.cuda.synchronize()
        for i in range(len(shapes)):
            assert torch.equal(plan.outs[i], refs[i]), (graph, i)
    plan.close()


def test_fold_in_batch_queue_mixed_and_nonfinite():
    """Folded instances run as queue tasks beside FFT levels and direct tiles;
    a non-finite input switches only its own instance to the tap-by-tap sums."""
    import torch
    from ndconv.batch import BatchPlan
    g = torch.Generator(device="cuda").manual_seed(7)
    shapes = [((300, 6, 5), (9, 21, 17)), ((100, 5, 4), (7, 15, 13)), ((100, 5, 4), (7, 15, 13)),
              ((150, 4, 9), (11, 13, 25)), ((200, 700), (11, 31)), ((64, 300), (5, 9))]
    algos = [0, 0, 0, 0, 1, 0]
    xs = [torch.rand(s, generator=g, device="cuda") for s, _ in shapes]
    ks = [torch.rand(k, generator=g, device="cuda") for _, k in shapes]
    xs[1][40, 2, 1] = float("inf")
    ks[2][3, 0, 12] = float("nan")
    kws = [with_dilation(k, 1) for k in ks]
    modes = [(_mode(k, 1, 1), PaddingMode.Reflect if i in (1, 2) else PaddingMode.Replicate)
             for i, (_, k) in enumerate(shapes)]
    plan = BatchPlan(modes, xs, kws, algos=algos)
    assert plan.info()["n_standalone"] == 0
    refs = [ndconv.conv_algo(xs[i], kws[i], *modes[i], algos[i]) for i in range(len(shapes))]
    for graph in (False, True):
        for y in plan.outs:
            y.fill_(-1.0)
        plan.run(graph=graph)
        plan.check()
        torch.cuda.synchronize()
        for i in range(len(shapes)):
            y, r = plan.outs[i].cpu().numpy(), refs[i].cpu().numpy()
            assert np.array_equal(np.isnan(y), np.isnan(r)) and np.array_equal(np.isinf(y), np.isinf(r)), (graph, i)
            if algos[i] == 0:
                assert np.array_equal(y, r, equal_nan=True), (graph, i)
            else:
                assert normwise_err(y, r) <= TOL32, (graph, i)
    for i in (1, 2):
        x64 = xs[i].double().cpu().numpy()
        k64 = ks[i].double().cpu().numpy()
        st, y64 = O.conv(problem(F64, x64, kws[i], *modes[i]), x64, k64)
        y = plan.outs[i].cpu().numpy()
        assert np.array_equal(np.isnan(y), np.isnan(y64)) and np.array_equal(np.isinf(y), np.isinf(y64))
    plan.close()
