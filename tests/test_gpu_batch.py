"""Heterogeneous batches: the persistent work-queue kernel (with and without
CUDA-graph replay) and the plain per-instance submission must give exactly
the per-instance entry points' results; one instance is also checked
against the f64 oracle."""
import numpy as np
import pytest

import ndconv
from helpers import F64, normwise_err, problem, with_dilation
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()


def _batch(n, seed, **kw):
    from ndconv import workloads as W
    specs = W.uneven_batch(n, seed=seed, **kw)
    xs, ks = W.make_tensors(specs, seed=seed)
    kws = [with_dilation(k, s.dilation) for k, s in zip(ks, specs)]
    modes = [(s.conv_mode(), s.padding_mode()) for s in specs]
    return specs, xs, ks, kws, modes


@pytest.mark.parametrize("seed", [1, 2])
def test_batch_matches_per_instance(seed):
    import torch
    from ndconv.batch import BatchPlan
    specs, xs, ks, kws, modes = _batch(60, seed, max_log2=14, kmax=31)
    rng = np.random.default_rng(seed)
    algos = [int(a) for a in rng.integers(0, 2, len(specs))]
    plan = BatchPlan(modes, xs, kws, algos=algos)
    info = plan.info()
    assert info["tasks"] > 0 and info["n_direct"] + info["n_fft"] + info["n_standalone"] == len(specs)
    refs = []
    for i, s in enumerate(specs):
        f = ndconv.conv if algos[i] == 0 else ndconv.conv_fft
        refs.append(f(xs[i], kws[i], *modes[i]))
    for form in ("queue", "graph", "graph2", "plain"):
        for y in plan.outs:
            y.fill_(float("nan"))
        if form == "plain":
            plan.run_plain()
        else:
            plan.run(graph=form != "queue")
        plan.check()
        torch.cuda.synchronize()
        for i in range(len(specs)):
            assert torch.equal(plan.outs[i], refs[i]), (form, i, specs[i], algos[i])
    # one instance against the f64 oracle
    i = int(np.argmax([np.prod(s.shape) for s in specs]))
    x, k = xs[i].cpu().numpy(), ks[i].cpu().numpy()
    p = problem(F64, x, with_dilation(k, specs[i].dilation), *modes[i])
    st, y64 = O.conv(p, x.astype(np.float64), k.astype(np.float64))
    assert st == 0
    assert normwise_err(plan.outs[i].cpu().numpy(), y64) <= 1e-5
    plan.close()


def test_batch_mixed_types_standalone():
    import torch
    from ndconv import BorderType, ConvMode, PaddingMode
    from ndconv.batch import BatchPlan
    g = torch.Generator(device="cuda").manual_seed(3)
    xs = [torch.rand((30, 40), generator=g, device="cuda", dtype=torch.float64),
          torch.randint(-9, 9, (50,), generator=g, device="cuda", dtype=torch.int32),
          torch.rand((8, 9, 10), generator=g, device="cuda")]
    ks = [torch.rand((3, 5), generator=g, device="cuda", dtype=torch.float64),
          torch.randint(-9, 9, (7,), generator=g, device="cuda", dtype=torch.int32),
          torch.rand((3, 3, 3), generator=g, device="cuda")]
    modes = [(ConvMode.Same, PaddingMode.Reflect), (ConvMode.Full, PaddingMode.Zeros),
             (ConvMode.Valid, PaddingMode.Custom([BorderType.Zeros] * 3))]
    algos = [1, 0, 1]
    plan = BatchPlan(modes, xs, ks, algos=algos)
    assert plan.info()["n_standalone"] == 2
    plan.run(graph=True)
    plan.check()
    for i in range(3):
        f = ndconv.conv if algos[i] == 0 else ndconv.conv_fft
        assert torch.equal(plan.outs[i], f(xs[i], ks[i], *modes[i]))
    plan.close()


@pytest.mark.parametrize("algo", [0, 1])
@pytest.mark.parametrize("dt", ["float32", "int32"])
def test_host_batch_equals_device_calls(algo, dt):
    import torch
    from helpers import BorderType, ConvMode, PaddingMode
    if algo == 1 and dt == "int32":
        pytest.skip("no integer FFT")
    g = torch.Generator().manual_seed(7)
    n, xs_, ks_ = 37, (64, 900), (5, 9)
    if dt == "int32":
        xs = [torch.randint(-100, 100, xs_, generator=g, dtype=torch.int32).pin_memory() for _ in range(n)]
        ks = [torch.randint(-9, 9, ks_, generator=g, dtype=torch.int32).pin_memory() for _ in range(n)]
    else:
        xs = [torch.rand(xs_, generator=g).pin_memory() for _ in range(n)]
        ks = [torch.rand(ks_, generator=g).pin_memory() for _ in range(n)]
    mode, pm = ConvMode.Same, PaddingMode.Custom([BorderType.Reflect, BorderType.Circular])
    ys = [torch.empty(xs_, dtype=xs[0].dtype).pin_memory() for _ in range(n)]
    ndconv.conv_batch_host(xs, [with_dilation(k, 2) for k in ks], ys, mode, pm, algo=algo)
    f = ndconv.conv if algo == 0 else ndconv.conv_fft
    for i in range(n):
        ref = f(xs[i].cuda(), with_dilation(ks[i].cuda(), 2), mode, pm).cpu()
        assert torch.equal(ys[i], ref), i


def test_batch_tensor_core_instances():
    """Instances sent to the tensor cores (algo 2) run beside the queue and
    give exactly what ndconv_conv_algo(NDCONV_ALGO_DIRECT_BF16X3) gives; an
    f64 instance given algo 2 runs the direct kernels."""
    import torch
    from ndconv import _abi, BorderType, ConvMode, PaddingMode
    from ndconv.batch import BatchPlan
    specs, xs, ks, kws, modes = _batch(24, 5, max_log2=14, kmax=31)
    algos = [2 if (s.rank >= 2 and i % 2 == 0) else (i % 2) for i, s in enumerate(specs)]
    g = torch.Generator(device="cuda").manual_seed(5)
    xs = list(xs) + [torch.rand((40, 60), generator=g, device="cuda", dtype=torch.float64),
                     torch.rand((70, 90), generator=g, device="cuda")]
    k64, k32 = (torch.rand((5, 7), generator=g, device="cuda", dtype=torch.float64),
                torch.rand((15, 17), generator=g, device="cuda"))
    kws = list(kws) + [with_dilation(k64, 1), with_dilation(k32, [1, 2])]
    ks = list(ks) + [k64, k32]
    modes = list(modes) + [(ConvMode.Same, PaddingMode.Reflect),
                           (ConvMode.Same, PaddingMode.Custom([BorderType.Circular, BorderType.Replicate]))]
    algos += [2, 2]
    assert sum(a == 2 for a in algos) >= 3
    plan = BatchPlan(modes, xs, kws, algos=algos)
    refs = []
    for i in range(len(xs)):
        if algos[i] == 2 and xs[i].dtype == torch.float32:
            refs.append(ndconv.conv_algo(xs[i], kws[i], *modes[i], _abi.ALGO_DIRECT_BF16X3))
        elif algos[i] in (0, 2):
            refs.append(ndconv.conv(xs[i], kws[i], *modes[i]))
        else:
            refs.append(ndconv.conv_fft(xs[i], kws[i], *modes[i]))
    for form in ("queue", "graph", "graph2", "plain"):
        for y in plan.outs:
            y.fill_(float("nan"))
        if form == "plain":
            plan.run_plain()
        else:
            plan.run(graph=form != "queue")
        plan.check()
        torch.cuda.synchronize()
        for i in range(len(xs)):
            assert torch.equal(plan.outs[i], refs[i]), (form, i, algos[i])
    # the last instance (tensor cores, dilation, mixed borders) against the f64 oracle
    x, k = xs[-1].cpu().numpy(), ks[-1].cpu().numpy()
    p = problem(F64, x, with_dilation(k, [1, 2]), *modes[-1])
    st, y64 = O.conv(p, x.astype(np.float64), k.astype(np.float64))
    assert st == 0
    assert normwise_err(plan.outs[-1].cpu().numpy(), y64) <= 1e-5
    plan.close()
