"""The uneven batch at its full benchmark size: 4096 instances (rank 1/2/3 =
60/35/5 %, 2^8..2^20 elements, odd kernels 3..127 per axis, dilation and
stride 1|2, Zeros/Reflect/Replicate/Circular) with the trained dispatcher's
picks (without the tensor-core variant), as the benchmark runs it.

* The persistent queue, its CUDA-graph replay and the plain per-instance
  submission give exactly (torch.equal) what the public per-instance entry
  points give, for every one of the 4096 instances.
* A stratified sample of >= 64 instances (every rank x border kind, the
  longest kernels, the tiniest axes under large pads) is within 1e-5
  normwise of the f64 oracle: its direct loop where that is cheap, its
  FFT convolution in f64 (the crate's conv_fft restated) elsewhere.
"""
import os

import numpy as np
import pytest

import ndconv
from helpers import F64, normwise_err, problem, with_dilation
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL32 = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()


@pytest.fixture(scope="module")
def batch():
    import torch
    from ndconv import workloads as W
    from ndconv.batch import BatchPlan
    from ndconv.mlp import MLPDispatcher, default_available
    specs = W.uneven_batch(4096, seed=4000)
    xs, ks = W.make_tensors(specs, seed=4000)
    kws = [with_dilation(k, s.dilation) for k, s in zip(ks, specs)]
    modes = [(s.conv_mode(), s.padding_mode()) for s in specs]
    # as the benchmark runs it: the tensor-core variant stays out of the
    # batch's picks (its launches beside the queue cost more than they save)
    avail = default_available()
    avail[1] = 0.0
    algos = [int(a) for a in MLPDispatcher(available=avail).choose(specs)]
    plan = BatchPlan(modes, xs, kws, algos=algos)
    yield specs, xs, ks, kws, modes, algos, plan
    plan.close()
    torch.cuda.synchronize()


def _per_instance(x, kw, mode, pm, algo):
    """The public per-instance call for the instance's pick.  A batch runs an
    instance whose FFT variant cannot take it (e.g. the full N-d form with
    rows longer than one CTA's shared memory) by the direct kernels, as
    ndconv_conv_fft does; the explicit variant call reports Unsupported."""
    if algo == 0:
        return ndconv.conv(x, kw, mode, pm)
    if algo == 1:
        return ndconv.conv_fft(x, kw, mode, pm)
    try:
        return ndconv.conv_algo(x, kw, mode, pm, algo)
    except ndconv.api.Unsupported:
        return ndconv.conv(x, kw, mode, pm)


def test_full_batch_equals_per_instance(batch):
    import torch
    specs, xs, ks, kws, modes, algos, plan = batch
    refs = [_per_instance(xs[i], kws[i], *modes[i], algos[i]) for i in range(len(specs))]
    torch.cuda.synchronize()
    for form in ("queue", "graph", "graph2", "plain"):
        for y in plan.outs:
            y.fill_(float("nan"))
        if form == "plain":
            plan.run_plain()
        else:
            plan.run(graph=form != "queue")
        plan.check()
        torch.cuda.synchronize()
        bad = [i for i in range(len(specs)) if not torch.equal(plan.outs[i], refs[i])]
        assert not bad, (form, len(bad), [(i, specs[i], algos[i]) for i in bad[:5]])


def _direct_cost(s):
    return float(np.prod(s.out_shape())) * float(np.prod(s.kshape))


def _oracle_ok(s):
    """the f64 oracle finishes in well under a second: its direct loop for
    at most 3e8 multiply-adds, else its FFT over at most 2e7 padded points"""
    fft_pts = float(np.prod([n + 2 * ((e - 1) // 2) for n, e in zip(s.shape, s.keff())]))
    return _direct_cost(s) < 3e8 or fft_pts <= 2e7


def _sample(specs, rng, algos):
    """>= 64 instances the oracle finishes: 4 per (rank, border kind), the 8
    longest kernels, the 8 tiniest axes relative to their dilated kernels,
    and up to 8 instances the dispatcher sent to the tensor cores."""
    pick = []
    tc = [i for i, a in enumerate(algos) if a == 2 and _oracle_ok(specs[i])]
    pick += [int(i) for i in rng.permutation(tc)[:8]]
    for rank in (1, 2, 3):
        for pad in ("Zeros", "Reflect", "Replicate", "Circular"):
            cand = [i for i, s in enumerate(specs) if s.rank == rank and s.pad == pad and _oracle_ok(s)]
            pick += [int(i) for i in rng.permutation(cand)[:4]]
    by_k = sorted(range(len(specs)), key=lambda i: -max(specs[i].keff()))
    pick += [i for i in by_k if i not in pick and _oracle_ok(specs[i])][:8]
    by_ratio = sorted(range(len(specs)), key=lambda i: min(n / e for n, e in zip(specs[i].shape, specs[i].keff())))
    pick += [i for i in by_ratio if i not in pick and _oracle_ok(specs[i])][:8]
    return pick


def test_full_batch_sample_vs_f64_oracle(batch):
    import torch
    specs, xs, ks, kws, modes, algos, plan = batch
    plan.run(graph=True)
    plan.check()
    torch.cuda.synchronize()
    sample = _sample(specs, np.random.default_rng(4096), algos)
    assert len(sample) >= 64
    # the sample reaches the regimes it is meant to cover
    assert max(max(specs[i].kshape) for i in sample) >= 121
    assert any(min(specs[i].shape) <= 8 and max(specs[i].keff()) >= 60 for i in sample)
    assert {specs[i].rank for i in sample} == {1, 2, 3}
    assert {algos[i] != 0 for i in sample} == {False, True}
    if any(a == 2 for a in algos):
        assert any(algos[i] == 2 for i in sample)
    nth = os.cpu_count() or 1
    for i in sample:
        s = specs[i]
        x = xs[i].cpu().numpy().astype(np.float64)
        k = ks[i].cpu().numpy().astype(np.float64)
        p = problem(F64, x, with_dilation(k, s.dilation), *modes[i])
        st, y64 = O.conv(p, x, k) if _direct_cost(s) < 3e8 else O.conv_fft(p, x, k, nth)
        assert st == 0, (i, s)
        y = plan.outs[i].cpu().numpy()
        assert y.shape == y64.shape, (i, s)
        err = normwise_err(y, y64)
        assert err <= TOL32, (i, s, algos[i], err)
