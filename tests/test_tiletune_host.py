"""CPU checks of the second-stage (tile / plan) tuning: the knobs are
thread-local host settings of the C ABI (set, read back, restored by the
context manager, unknown knobs refused), and the nearest-neighbour knob
picker and its regret accounting behave on a synthetic timing set.  No
device work."""
import threading

import numpy as np
import pytest

from ndconv import _abi
from ndconv import tiletune as TT


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()


def test_knobs_are_thread_local_and_restored():
    L = _abi.lib()
    assert L.ndconv_get_tuning(_abi.TUNE_MAC_ROWS) == 0
    with TT.tuning({_abi.TUNE_MAC_ROWS: 4, _abi.TUNE_SW_TY: 2}):
        assert L.ndconv_get_tuning(_abi.TUNE_MAC_ROWS) == 4
        assert L.ndconv_get_tuning(_abi.TUNE_SW_TY) == 2
        seen = []
        t = threading.Thread(target=lambda: seen.append(L.ndconv_get_tuning(_abi.TUNE_MAC_ROWS)))
        t.start()
        t.join()
        assert seen == [0]  # another thread keeps the library's choice
    assert L.ndconv_get_tuning(_abi.TUNE_MAC_ROWS) == 0
    assert L.ndconv_get_tuning(_abi.TUNE_SW_TY) == 0
    assert L.ndconv_set_tuning(99, 1) == _abi.ERR_INVALID
    assert L.ndconv_set_tuning(_abi.TUNE_SW_TY, -1) == _abi.ERR_INVALID


def test_knob_space_shape():
    assert TT.ALGOS == [0, 2, 3, 4, 5, 6]
    for _, combos in TT.KNOB_SPACE:
        assert combos[0] == {}  # the library's own choice comes first
        assert len(combos) <= TT.MAX_COMBOS


def _synthetic(n, rng):
    """two feature clusters; in each, a different combination of variant 0 is best"""
    F = rng.standard_normal((n, 16))
    F[: n // 2, :12] += 8
    T = np.full((n, len(TT.ALGOS), TT.MAX_COMBOS), np.inf)
    T[:, :, :3] = 10.0
    T[: n // 2, 0, 1] = 4.0   # cluster A: combination 1
    T[n // 2:, 0, 2] = 5.0    # cluster B: combination 2
    T[:, 1, 0] = 20.0         # variant 1 slower everywhere
    return F, T


def test_picker_finds_each_clusters_combination():
    rng = np.random.default_rng(0)
    F, T = _synthetic(400, rng)
    picker = TT.KnobPicker(F, T, k=8)
    Fq, _ = _synthetic(40, np.random.default_rng(1))
    assert all(picker.pick(Fq[i], 0) == 1 for i in range(20))
    assert all(picker.pick(Fq[i], 0) == 2 for i in range(20, 40))


def test_evaluate_accounts_regret():
    rng = np.random.default_rng(2)
    F, T = _synthetic(200, rng)
    picker = TT.KnobPicker(F, T, k=8)
    Fh, Th = _synthetic(50, np.random.default_rng(3))
    rep = TT.evaluate(picker, Fh, Th, [TT.ALGOS[0]] * 50)
    assert rep["first_stage_tuned_knobs"]["total_ratio"] == pytest.approx(1.0)
    assert rep["first_stage_default_knobs"]["total_ratio"] > 2.0
    assert rep["sum_ms"]["tuned_knobs"] <= rep["sum_ms"]["default_knobs"]


@pytest.mark.gpu  # the first stage's network runs on the library's CUDA kernels
def test_shipped_two_stage_dispatcher_picks_valid_settings():
    from ndconv import workloads as W
    d = TT.TwoStageDispatcher()
    specs = W.uneven_batch(20, seed=11)
    picks = d.choose(specs)
    assert len(picks) == 20
    for algo, settings in picks:
        ai = TT.ALGOS.index(algo)
        assert settings in TT.KNOB_SPACE[ai][1]
