"""Failure reporting without a GPU fault.

* The persistent queue's dependency waits are bounded.  With a short poll
  bound and one task made to wait on a counter that no task bumps, the wait
  runs out: the kernel still returns, ndconv_batch_status reports
  NDCONV_ERR_TIMEOUT, and the same plan at the default bound runs clean and
  gives the per-instance results again.
* The 3xBF16 tensor-core path keeps its (never expected) timeouts in a
  per-device word: after ordinary runs ndconv_bf16x3_status reports none.
"""
import ctypes

import pytest

import ndconv
from helpers import BorderType, ConvMode, PaddingMode, with_dilation
from ndconv import _abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__ as g
    g.build()


def _fft_batch():
    import torch
    from ndconv.batch import BatchPlan
    g = torch.Generator(device="cuda").manual_seed(11)
    shapes = [(60, 900), (40, 700), (9, 30, 50), (300,)]
    kshapes = [(5, 9), (7, 3), (3, 5, 5), (17,)]
    xs = [torch.rand(s, generator=g, device="cuda") for s in shapes]
    ks = [torch.rand(s, generator=g, device="cuda") for s in kshapes]
    kws = [with_dilation(k, 2) for k in ks]
    modes = [(ConvMode.Same, PaddingMode.Custom([BorderType.Reflect] * len(s))) for s in shapes]
    plan = BatchPlan(modes, xs, kws, algos=[1] * len(xs))
    refs = [ndconv.conv_fft(x, kw, *m) for x, kw, m in zip(xs, kws, modes)]
    return plan, refs


@pytest.mark.parametrize("graph", [False, True])
def test_queue_wait_runs_out_and_is_reported(graph):
    import torch
    plan, refs = _fft_batch()
    assert plan.info()["n_fft"] >= 3  # FFT instances inside the queue: tasks that wait on levels
    plan.run(graph=graph)
    assert plan.status() == _abi.OK
    # one wait that can never be satisfied, a short bound: the wait gives up
    plan.set_wait_limit(200)
    plan.stall_one_wait(True)
    plan.run(graph=graph)
    assert plan.status() == _abi.ERR_TIMEOUT
    assert "waited too long" in _abi.last_error()
    # the same plan, restored, at the default bound
    plan.stall_one_wait(False)
    plan.set_wait_limit(0)
    for y in plan.outs:
        y.fill_(float("nan"))
    plan.run(graph=graph)
    assert plan.status() == _abi.OK
    torch.cuda.synchronize()
    for y, r in zip(plan.outs, refs):
        assert torch.equal(y, r)
    plan.close()


def test_bf16x3_status_clean_after_runs():
    import torch
    L = _abi.lib()
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.ndconv_bf16x3_status(sp) == _abi.OK  # clears anything earlier tests left
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.rand((6, 40, 300), generator=g, device="cuda")
    k = torch.rand((3, 5, 31), generator=g, device="cuda")
    y = ndconv.conv_algo(x, k, ConvMode.Same, PaddingMode.Zeros, _abi.ALGO_DIRECT_BF16X3)
    assert torch.isfinite(y).all()
    assert L.ndconv_bf16x3_status(sp) == _abi.OK
