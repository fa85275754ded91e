"""Tile and plan tuning inside each algorithm: the second stage of the
dispatcher.

The first stage (ndconv.mlp) picks the algorithm variant of an instance.
Inside a variant the library exposes tile / plan knobs (ndconv_set_tuning):
row sets per CTA and rows per warp line of the sliding-window direct kernel,
output rows per CTA of the
FFT spectral tap sum and threads of the FFT row passes, and the tensor-core
tile width.  This module times every knob combination of every variant on a
set of configurations (CUDA events, warm-up, best of `reps`), keeps the
timings, and picks knobs for a new instance from its nearest timed
neighbours in feature space (the geometric mean of each combination's
slow-down against each neighbour's best).  Its picks are judged by regret
against the exhaustive search over all (variant, knobs) pairs.

    python -m ndconv.tiletune --train 2500 --holdout 500 --out DIR
"""
import argparse
import contextlib
import ctypes
import json
import math
import os
import time

import numpy as np

from . import _abi
from .api import build_problem, with_dilation

# (variant, [knob settings]) -- settings are {knob: value}; {} is the library's choice
KNOB_SPACE = [
    (_abi.ALGO_DIRECT, [{}] + [{_abi.TUNE_SW_TY: t, _abi.TUNE_SW_RY: r} for t in (1, 2, 4, 8) for r in (1, 2, 4)]),
    (_abi.ALGO_DIRECT_BF16X3, [{}] + [{_abi.TUNE_BF16X3_BN: b} for b in (16, 32, 64)]),
    (_abi.ALGO_FFT_ND, [{}] + [{_abi.TUNE_ROW_THREADS: t} for t in (128, 256, 512)]),
    (_abi.ALGO_FFT_RS, [{_abi.TUNE_MAC_ROWS: m, _abi.TUNE_ROW_THREADS: t} if (m or t) else {}
                        for m in (0, 1, 2, 4) for t in (0, 256, 512)]),
    (_abi.ALGO_FFT_ND_POW2, [{}] + [{_abi.TUNE_ROW_THREADS: t} for t in (128, 256, 512)]),
    (_abi.ALGO_FFT_RS_POW2, [{_abi.TUNE_MAC_ROWS: m, _abi.TUNE_ROW_THREADS: t} if (m or t) else {}
                             for m in (0, 1, 2, 4) for t in (0, 256, 512)]),
]
ALGOS = [a for a, _ in KNOB_SPACE]
MAX_COMBOS = max(len(c) for _, c in KNOB_SPACE)


@contextlib.contextmanager
def tuning(settings):
    """Apply knob settings on this thread for the duration of the block."""
    L = _abi.lib()
    old = {k: L.ndconv_get_tuning(k) for k in settings}
    try:
        for k, v in settings.items():
            if L.ndconv_set_tuning(int(k), int(v)):
                raise RuntimeError(_abi.last_error())
        yield
    finally:
        for k, v in old.items():
            L.ndconv_set_tuning(int(k), int(v))


class KnobTimes:
    """spec -> times [len(ALGOS), MAX_COMBOS] in ms (inf: combination
    unavailable for the instance, or padding)."""

    def __init__(self):
        self.specs, self.times = [], []

    def add(self, spec, t):
        self.specs.append(spec)
        self.times.append(np.asarray(t, np.float64))

    def array(self):
        return np.array(self.times, np.float64).reshape(len(self.times), len(ALGOS), MAX_COMBOS)

    def save(self, path):
        from .workloads import PAD_MODES
        S = self.specs
        np.savez_compressed(
            path, rank=np.array([s.rank for s in S], np.int8),
            shape=np.array([list(s.shape) + [1] * (3 - s.rank) for s in S], np.int32),
            kshape=np.array([list(s.kshape) + [1] * (3 - s.rank) for s in S], np.int16),
            misc=np.array([[s.dilation, s.stride, PAD_MODES.index(s.pad)] for s in S], np.int8),
            times=self.array().astype(np.float32), algos=np.array(ALGOS, np.int8))

    @classmethod
    def load(cls, path):
        from .workloads import PAD_MODES, Spec
        z = np.load(path)
        db = cls()
        for r, sh, ks, mi, t in zip(z["rank"], z["shape"], z["kshape"], z["misc"], z["times"]):
            r = int(r)
            db.add(Spec([int(v) for v in sh[:r]], [int(v) for v in ks[:r]], int(mi[0]), int(mi[1]),
                        PAD_MODES[int(mi[2])]), t.astype(np.float64))
        return db


def time_spec(spec, gen, reps=2, only=None):
    """[len(ALGOS), MAX_COMBOS] best-of-reps times (ms) of one instance
    (variants outside `only`, when given, stay inf)."""
    import torch
    L = _abi.lib()
    x = torch.rand(spec.shape, generator=gen, device="cuda") * 2 - 1
    k = torch.rand(spec.kshape, generator=gen, device="cuda") * 2 - 1
    p = build_problem(_abi.F32, spec.shape, with_dilation(k, spec.dilation), spec.conv_mode(),
                      spec.padding_mode())
    y = torch.empty(spec.out_shape(), device="cuda")
    st = torch.cuda.current_stream()
    sp = ctypes.c_void_p(st.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = np.full((len(ALGOS), MAX_COMBOS), np.inf)
    for ai, (algo, combos) in enumerate(KNOB_SPACE):
        if only is not None and algo not in only:
            continue
        for ci, settings in enumerate(combos):
            with tuning(settings):
                call = (ctypes.byref(p), algo, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(k.data_ptr()),
                        ctypes.c_void_p(y.data_ptr()), sp)
                if L.ndconv_conv_algo(*call) != 0:
                    break  # the variant does not take this instance
                best = math.inf
                for _ in range(reps):
                    e0.record(st)
                    L.ndconv_conv_algo(*call)
                    e1.record(st)
                    e1.synchronize()
                    best = min(best, e0.elapsed_time(e1))
                out[ai, ci] = best
    torch.cuda.synchronize()
    return out


class KnobPicker:
    """Second stage: knobs for (instance, variant) from the k nearest timed
    configurations (standardised features) on which the variant ran."""

    def __init__(self, feats, times, k=8):
        self.F = np.asarray(feats, np.float64)
        self.mu, self.sd = self.F.mean(0), self.F.std(0) + 1e-9
        self.Z = (self.F - self.mu) / self.sd
        self.T = np.asarray(times, np.float64)  # [n, algos, combos]
        self.k = k

    def pick(self, feat, ai):
        """combination index for variant ALGOS[ai]"""
        t = self.T[:, ai, :]
        best = t.min(1)
        ok = np.isfinite(best)
        if not ok.any():
            return 0
        z = (np.asarray(feat, np.float64) - self.mu) / self.sd
        d = ((self.Z[ok] - z) ** 2).sum(1)
        nn = np.argsort(d)[: self.k]
        rel = t[ok][nn] / best[ok][nn][:, None]
        score = np.where(np.isfinite(rel), np.log(rel), np.inf).mean(0)
        return int(np.argmin(score))


DEFAULT_TIMINGS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "knob_timings.npz")


class TwoStageDispatcher:
    """First stage: the trained network's variant; second stage: the knob
    settings the nearest timed configurations favour for that variant.
    choose(specs) -> [(ndconv_algo, {knob: value})]; run an instance with
    `with tuning(settings): ndconv.conv_algo(x, k, mode, pm, algo)`."""

    def __init__(self, timings=DEFAULT_TIMINGS, k=8):
        from .dispatch import features
        from .mlp import MLPDispatcher
        db = KnobTimes.load(timings)
        self.picker = KnobPicker(np.array([features(s) for s in db.specs]), db.array(), k=k)
        self.first = MLPDispatcher()

    def choose(self, specs):
        from .dispatch import features
        out = []
        for s, a in zip(specs, self.first.choose(specs)):
            ai = ALGOS.index(int(a))
            c = self.picker.pick(features(s), ai)
            out.append((int(a), dict(KNOB_SPACE[ai][1][c])))
        return out


def evaluate(picker, feats, times, algo_picks):
    """Regret against the exhaustive search over (variant, knobs):
    the first-stage variant with the library's knobs, with the second-stage
    knobs, with the best knobs of that variant, and the best pair."""
    from .autotune import regret
    T = np.asarray(times, np.float64)
    n = len(T)
    best_all = T.reshape(n, -1).min(1)
    t_default, t_tuned, t_bestknob = [], [], []
    for i in range(n):
        ai = ALGOS.index(algo_picks[i])
        row = T[i, ai]
        if not np.isfinite(row[0]):
            ai = int(np.argmin(T[i].min(1)))  # the first-stage pick could not run: its fallback
            row = T[i, ai]
        t_default.append(row[0])
        c = picker.pick(feats[i], ai)
        t_tuned.append(row[c] if np.isfinite(row[c]) else row[0])
        t_bestknob.append(row.min())
    return {"n": n,
            "first_stage_default_knobs": regret(t_default, best_all),
            "first_stage_tuned_knobs": regret(t_tuned, best_all),
            "first_stage_best_knobs": regret(t_bestknob, best_all),
            "sum_ms": {"best_pair": float(best_all.sum()), "default_knobs": float(np.sum(t_default)),
                       "tuned_knobs": float(np.sum(t_tuned)), "best_knobs": float(np.sum(t_bestknob))}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2500)
    ap.add_argument("--holdout", type=int, default=500)
    ap.add_argument("--seed", type=int, default=7000)
    ap.add_argument("--out", required=True)
    ap.add_argument("--timings", default=None, help="reuse saved knob timings")
    ap.add_argument("--retime-algo", type=int, default=None,
                    help="with --timings: time this variant's knob settings again")
    ap.add_argument("--retime-rank", type=int, nargs="*", default=[1, 2, 3],
                    help="ranks whose instances --retime-algo times again")
    args = ap.parse_args()
    import torch
    from .autotune import dispatcher_configs
    from .dispatch import features
    from .mlp import MLPDispatcher
    os.makedirs(args.out, exist_ok=True)
    t0 = time.time()
    if args.timings:
        db = KnobTimes.load(args.timings)
        if args.retime_algo is not None:
            ai = ALGOS.index(args.retime_algo)
            gen = torch.Generator(device="cuda").manual_seed(args.seed)
            for i, s in enumerate(db.specs):
                if s.rank in args.retime_rank:
                    db.times[i][ai] = time_spec(s, gen, only=(args.retime_algo,))[ai]
            db.save(os.path.join(args.out, "knob_timings.npz"))
    else:
        specs = dispatcher_configs(args.train + args.holdout, seed=args.seed)
        gen = torch.Generator(device="cuda").manual_seed(args.seed)
        db = KnobTimes()
        for i, s in enumerate(specs):
            db.add(s, time_spec(s, gen))
            if (i + 1) % 500 == 0:
                print(f"timed {i + 1}/{len(specs)} in {time.time() - t0:.0f} s", flush=True)
        db.save(os.path.join(args.out, "knob_timings.npz"))
    t_tune = time.time() - t0
    T = db.array()
    F = np.array([features(s) for s in db.specs])
    ntr = args.train
    picker = KnobPicker(F[:ntr], T[:ntr])
    disp = MLPDispatcher()
    algo_picks = disp.choose(db.specs[ntr:])
    rep = {"train": ntr, "holdout": len(db.specs) - ntr, "tune_s": t_tune,
           "knob_space": [[int(a), [{str(k): v for k, v in c.items()} for c in cs]] for a, cs in KNOB_SPACE],
           "holdout_eval": evaluate(picker, F[ntr:], T[ntr:], algo_picks)}
    with open(os.path.join(args.out, "tile_tuning_report.json"), "w") as f:
        json.dump(rep, f, indent=1)
    print(json.dumps(rep["holdout_eval"]), flush=True)


if __name__ == "__main__":
    main()
