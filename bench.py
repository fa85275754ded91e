"""Benchmark: convolution GB/s and % of HBM roofline on one GB300.

Headline workload (the reference's 2-D benchmark case, batched): B = 64
independent instances of a 2-D f32 convolution x[200, 5000] with a kernel
[11, 31] dilated by 2, ConvMode::Same, PaddingMode::Custom([Reflect,
Circular]); every instance has its own seeded Uniform[0,1) data and kernel
(numpy PCG64, seed 1000 + rank, the same instances in both arms).  A step is
one pass of conv_fft over all B instances.  B = 64 makes the inputs (256 MB)
larger than L2, so no flush is needed.

Metric: algorithmic bytes 4 * (|x| + |k| + |y|) per instance / time.
  value   device-resident inputs, CUDA-event timed (max over ranks)
  e2e     the library's host-memory batch entry point: pinned-host inputs,
          H2D copy + conv + D2H of the outputs inside the timed region
The default line also carries, in `config`:
  direct        the same 64 instances through conv (direct FP32), with its
                FP32 FMA roofline and the i32 copy's bit-exactness
  uneven_batch  the uneven batch (4096 instances, one persistent launch +
                CUDA graph, dispatcher-picked variants) against the plain
                drop-in (per-instance calls with the library's default picks)
  direct_tensor_cores  the same 64 instances through the batched 3xBF16
                tensor-core direct path (one persistent launch)
  replicated    configs 1 and 3 as 64-instance batches through the batched
                FFT, direct FP32 and tensor-core entry points
  variants      the 1-D and 3-D cases (and the 3-D complex copy, and a 2-D
                31 x 31 kernel) through direct FP32, 3xBF16 tensor cores
                and FFT: device time per call and error against f64
Reference arm (--impl reference): the oracle port of conv_fft_par (same
algorithm as the crate, rayon-style threads on all host cores) over the
same 64 instances per step.  The GPU line's cpu_baseline is that arm run as
a fresh process for ~--cpu-seconds.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "ndarray-conv_gb300")]

import numpy as np  # noqa: E402

# DRAM bytes (read + write) per instance of the batched FFT path, from one
# ncu capture of the timed workload: one 64-instance wave (the two row-pass
# launches of one step), profiles/conv_fft_2d_200x5000_k11x31_batch64_traffic.md
PROFILED_TRAFFIC = {"fft": 17.594e6}
PROFILED_TRAFFIC_SOURCE = "profiles/conv_fft_2d_200x5000_k11x31_batch64_traffic.md"

# the benchmark's metric; every line (both arms, both workloads) reports it
METRIC = "conv GB/s & % HBM roofline, batched+tuned vs plain GPU, err ≤1e-5 vs FP64"
METRIC_DETAIL = "GB/s of algorithmic bytes 4*(|x|+|k|+|y|) per instance"

SHAPE_X = (200, 5000)
SHAPE_K = (11, 31)
DIL = 2
SEED_C2 = 1000  # + rank
WORKLOAD_C2 = ("{B} x 2-D f32 x[200,5000] * k[11,31] dilation 2, Same, Custom([Reflect, Circular]); "
               "{what}, {form} submission")


def c2_inputs(B, seed, dtype=np.float32):
    """The headline workload's instances: B seeded Uniform[0,1) data and
    kernels (i32: Uniform{-100..100}), identical in both arms."""
    rng = np.random.default_rng(seed)
    if dtype == np.int32:
        xs = [rng.integers(-100, 101, SHAPE_X, dtype=np.int32) for _ in range(B)]
        ks = [rng.integers(-100, 101, SHAPE_K, dtype=np.int32) for _ in range(B)]
    else:
        xs = [rng.random(SHAPE_X, dtype=np.float32) for _ in range(B)]
        ks = [rng.random(SHAPE_K, dtype=np.float32) for _ in range(B)]
    return xs, ks


def algorithmic_bytes(out_shape):
    return 4 * (np.prod(SHAPE_X) + np.prod(SHAPE_K) + np.prod(out_shape))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def fp32_fma_roofline(out_shape, ms_per_instance, sm_mhz=None):
    """The direct path's compute roofline: 2 |y| nnz(k) flops per instance
    (the taps of the 2-D case are all non-zero) against the CUDA cores' FP32
    FMA peak, 152 SMs x 128 lanes x 2 flops x the SM clock (the measured
    maximum unless a sampled clock is given)."""
    flops = 2.0 * float(np.prod(out_shape)) * float(np.prod(SHAPE_K))
    mhz = sm_mhz
    if not mhz:
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                mhz = float(json.load(f)["sm_max_mhz"])
        except Exception:
            mhz = 2070.0
    peak = 152 * 128 * 2 * mhz * 1e6 / 1e12
    achieved = flops / (ms_per_instance * 1e-3) / 1e12
    return {"bound": "fp32_fma", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "flops_per_instance": flops}


def problem_args():
    import ndconv
    from ndconv import BorderType, ConvMode, PaddingMode
    return ConvMode.Same, PaddingMode.Custom([BorderType.Reflect, BorderType.Circular]), ndconv


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(seconds, batch):
    """The reference arm (the oracle port of conv_fft_par over the same
    instances) run as a fresh process for ~`seconds`, so that its figure is
    the arm's own and no thread of this GPU process competes for the cores."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1000000",
           "--warmup", "1", "--batch", str(batch), "--ref-seconds", str(seconds)]
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=600)
    if r.returncode:
        return None
    line = json.loads(r.stdout.strip().splitlines()[-1])
    cb = dict(line["cpu_baseline"])
    cb["value"] = line["value"]
    return cb


def run_reference(args, rank, world):
    """The reference arm: the oracle port of conv_fft_par (threads on all
    host cores) over the headline workload's instances, each step one pass
    over all of them.  Rank 0 only."""
    if rank != 0:
        return
    steps, warm = args.steps, args.warmup
    from oracle import oracle as O
    from ndconv import _abi, build_problem, with_dilation
    mode, pm, _ = problem_args()
    nth = os.cpu_count() or 1
    B = args.batch
    xs, ks = c2_inputs(B, SEED_C2)
    p = build_problem(_abi.F32, SHAPE_X, with_dilation(ks[0], DIL), mode, pm)
    for w in range(max(1, warm)):
        st, y = O.conv_fft(p, xs[w % B], ks[w % B], nth)
        assert st == 0
    t0 = time.perf_counter()
    done = 0
    for _ in range(steps):
        for i in range(B):
            O.conv_fft(p, xs[i], ks[i], nth)
        done += 1
        if args.ref_seconds and time.perf_counter() - t0 >= args.ref_seconds:
            break
    el = time.perf_counter() - t0
    gbs = algorithmic_bytes(y.shape) * B * done / el / 1e9
    sample = (f"{B} distinct instances of x[200,5000]*k[11,31] per step, {done} step(s) in {el:.1f} s "
              f"(conv_fft_par port, f32)")
    line = {"metric": METRIC,
            "value": gbs, "unit": "GB/s", "n_gpus": world, "steps": done, "warmup": warm,
            "ms_per_step": el / done * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": f"synthetic (seeded Uniform[0,1), distinct data and kernel per instance, seed {SEED_C2})",
            "impl": "reference",
            "config": {"workload": WORKLOAD_C2.format(B=B, what="conv_fft", form="batched"),
                       "metric_detail": METRIC_DETAIL, "batch_per_gpu": B},
            "cpu_baseline": {"value": gbs, "unit": "GB/s", "cores": nth, "kind": "port", "sample": sample},
            "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def flat_views(shapes, dtype, device):
    """One flat buffer and per-instance views into it."""
    import math
    import torch
    sizes = [math.prod(s) for s in shapes]
    buf = torch.empty(sum(sizes), dtype=dtype, device=device)
    views, off = [], 0
    for s, n in zip(shapes, sizes):
        views.append(buf[off:off + n].view(*s))
        off += n
    return buf, views


def measure_uneven(args, world, rank, local_rank, dist):
    """The uneven batch: independent instances in one persistent
    launch (device work queue, CUDA graph), against the same instances
    through the per-instance entry points (the plain drop-in).  Returns the
    figures of this rank (times max-reduced over ranks)."""
    import torch
    from ndconv import _abi, with_dilation
    from ndconv import workloads as W
    from ndconv import shard
    from ndconv.batch import BatchPlan
    from ndconv.dispatch import ModelDispatcher
    L = _abi.lib()
    # one batch of n instances per rank, split across ranks by estimated cost
    # (no data exchange between ranks)
    specs_all = W.uneven_batch(args.n_instances * world, seed=4000)
    specs = [specs_all[i] for i in shard.local_share(specs_all, rank, world)]
    gen = torch.Generator(device="cuda").manual_seed(4000 + rank)
    xbuf, xs = flat_views([s.shape for s in specs], torch.float32, "cuda")
    kbuf, ks = flat_views([s.kshape for s in specs], torch.float32, "cuda")
    ybuf, ys = flat_views([tuple(s.out_shape()) for s in specs], torch.float32, "cuda")
    xbuf.uniform_(-1, 1, generator=gen)
    kbuf.uniform_(-1, 1, generator=gen)
    if args.dispatch == "mlp":
        from ndconv.mlp import MLPDispatcher, default_available
        # the tensor-core variant runs beside the queue as ordinary launches
        # that want every SM's shared memory; measured on this batch it only
        # costs (71 ms per step without it, 112 ms with its 87 largest picks)
        avail = default_available()
        avail[1] = 0.0
        algos = MLPDispatcher(available=avail).choose(specs)
    else:
        algos = ModelDispatcher().choose(specs)
    plan = BatchPlan([(s.conv_mode(), s.padding_mode()) for s in specs], xs,
                     [with_dilation(k, s.dilation) for k, s in zip(ks, specs)], outs=ys, algos=algos)
    info = plan.info()
    stream = torch.cuda.current_stream()

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    plan.run(graph=False)  # first run outside capture (kernel attributes, tables)
    for _ in range(args.warmup):
        plan.run(graph=True)
    plan.check()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = L.ndconv_kernel_launches()
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            plan.run(graph=True)
        e1.record(stream)
        barrier()
    launches = L.ndconv_kernel_launches() - n0
    ms = e0.elapsed_time(e1) / args.steps
    plan.check()
    # plain per-instance entry points, same algorithms
    plan.run_plain()
    barrier()
    e0.record(stream)
    nplain = max(1, args.steps // 2)
    for _ in range(nplain):
        plan.run_plain()
    e1.record(stream)
    barrier()
    plain_ms = e0.elapsed_time(e1) / nplain
    # the plain drop-in: the same instances as per-instance library calls with
    # the library's default choice (cost model), no batching, no tuning
    dropin_ms = plain_ms
    if args.dispatch != "model":
        dplan = BatchPlan([(s.conv_mode(), s.padding_mode()) for s in specs], xs,
                          [with_dilation(k, s.dilation) for k, s in zip(ks, specs)], outs=ys,
                          algos=ModelDispatcher().choose(specs))
        dplan.run_plain()
        barrier()
        e0.record(stream)
        for _ in range(nplain):
            dplan.run_plain()
        e1.record(stream)
        barrier()
        dropin_ms = e0.elapsed_time(e1) / nplain
        dplan.close()
        plan.run(graph=True)  # outputs of the measured plan again (spot checks below)
        barrier()
    # end to end: inputs from pinned host memory, outputs back to it
    hx, hk = xbuf.cpu().pin_memory(), kbuf.cpu().pin_memory()
    hy = torch.empty_like(ybuf, device="cpu").pin_memory()
    for _ in range(2):
        xbuf.copy_(hx, non_blocking=True)
        kbuf.copy_(hk, non_blocking=True)
        plan.run(graph=True)
        hy.copy_(ybuf, non_blocking=True)
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        xbuf.copy_(hx, non_blocking=True)
        kbuf.copy_(hk, non_blocking=True)
        plan.run(graph=True)
        hy.copy_(ybuf, non_blocking=True)
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    if dist:
        t = torch.tensor([ms, plain_ms, e2e_ms, dropin_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, plain_ms, e2e_ms, dropin_ms = [float(v) for v in t.tolist()]
    bytes_step = sum(s.bytes() for s in specs)
    # parity spot checks against the f64 oracle: a seeded sample of direct and
    # FFT instances (the f64 FFT oracle where the direct loop is too slow)
    from oracle import oracle as O
    from ndconv import build_problem
    errs = []
    rng = np.random.default_rng(99)
    for want in (0, 1):
        cand = [i for i in range(len(specs)) if (algos[i] != 0) == bool(want)]
        for i in rng.permutation(cand)[:4]:
            i = int(i)
            s = specs[i]
            x0, k0 = xs[i].cpu().numpy().astype(np.float64), ks[i].cpu().numpy().astype(np.float64)
            p = build_problem(_abi.F64, s.shape, with_dilation(k0, s.dilation), s.conv_mode(), s.padding_mode())
            cost = float(np.prod(s.out_shape())) * float(np.prod(s.kshape))
            st, y64 = O.conv(p, x0, k0) if cost < 3e8 else O.conv_fft(p, x0, k0, os.cpu_count() or 1)
            if st == 0:
                y = ys[i].cpu().numpy().astype(np.float64)
                errs.append(float(np.linalg.norm(y - y64) / max(np.linalg.norm(y64), 1e-300)))
    plan.close()
    return {"specs": specs, "algos": algos, "info": info, "ms": ms, "plain_ms": plain_ms, "dropin_ms": dropin_ms,
            "e2e_ms": e2e_ms, "bytes_step": bytes_step, "launches": int(launches), "clocks": clk.summary(),
            "err": max(errs) if errs else None, "n_checked": len(errs),
            "h2d": int((xbuf.numel() + kbuf.numel()) * 4), "d2h": int(ybuf.numel() * 4),
            "x_gb": xbuf.numel() * 4 / 1e9}


def uneven_summary(r, world):
    """The uneven batch's figures, as the headline line's config.uneven_batch."""
    def gbs(ms):
        return r["bytes_step"] * world / (ms * 1e-3) / 1e9
    return {"workload": f"uneven batch: {len(r['specs'])} instances per GPU (rank 1/2/3 = 60/35/5%, "
                        "2^8..2^20 elements, odd kernels 3..127, dilation/stride 1|2, "
                        "Zeros/Reflect/Replicate/Circular), one persistent launch + CUDA graph",
            "batched_gbs": gbs(r["ms"]), "ms_per_step": r["ms"],
            "plain_per_instance_gbs": gbs(r["plain_ms"]), "batched_over_plain": r["plain_ms"] / r["ms"],
            "plain_dropin_gbs": gbs(r["dropin_ms"]), "batched_tuned_over_plain_dropin": r["dropin_ms"] / r["ms"],
            "e2e_gbs": gbs(r["e2e_ms"]), "normwise_err": r["err"], "err_checked_instances": r["n_checked"],
            "algos": {"direct": int(sum(a == 0 for a in r["algos"])), "fft": int(sum(a != 0 for a in r["algos"]))},
            "plan": r["info"], "gpu_launches": r["launches"], "clocks": r["clocks"],
            "plain_note": "plain = per-instance calls with the same picks; plain drop-in = "
                          "per-instance calls with the library's default (cost model) picks"}


def bench_uneven(args, world, rank, local_rank, dist):
    """--config c4: the uneven batch as the line's own workload."""
    r = measure_uneven(args, world, rank, local_rank, dist)
    if rank != 0:
        return
    peak, peak_kind = peaks()
    cpu = None
    if not args.no_cpu_baseline and world == 1:  # host-core baseline at N = 1 only
        cpu = cpu_baseline_uneven(r["specs"], args.cpu_seconds)
    u = uneven_summary(r, world)
    achieved = r["bytes_step"] / (r["ms"] * 1e-3) / 1e9
    line = {
        "metric": METRIC,
        "value": u["batched_gbs"], "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded; uneven-batch distribution)",
        "config": dict(u, metric_detail=METRIC_DETAIL, instances_per_gpu=len(r["specs"]),
                       dispatcher={"mlp": "trained network (ndconv/data/dispatcher_mlp.json)",
                                   "model": "cost model"}[args.dispatch],
                       l2=f"inputs {r['x_gb']:.2f} GB per GPU, larger than L2, no flush"),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "persistent batch kernel (one launch per step, plus standalone launches)",
                     "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
        "cpu_baseline": cpu,
        "e2e": {"value": u["e2e_gbs"], "unit": "GB/s", "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"]},
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "normwise_err_vs_f64": r["err"],
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_uneven(specs, seconds):
    """The oracle port of conv_fft_par on host cores over a seeded sample of
    the batch's instances, for ~`seconds`."""
    from oracle import oracle as O
    from ndconv import _abi, build_problem, with_dilation
    nth = os.cpu_count() or 1
    rng = np.random.default_rng(7)
    order = rng.permutation(len(specs))
    done_bytes, n, t0 = 0, 0, time.perf_counter()
    for i in order:
        s = specs[i]
        if np.prod(s.shape) * np.prod([k * s.dilation for k in s.kshape]) > 5e9:
            continue  # keep the sample bounded
        x = rng.uniform(-1, 1, s.shape).astype(np.float32)
        k = rng.uniform(-1, 1, s.kshape).astype(np.float32)
        p = build_problem(_abi.F32, s.shape, with_dilation(k, s.dilation), s.conv_mode(), s.padding_mode())
        st, _ = O.conv_fft(p, x, k, nth)
        if st == 0:
            done_bytes += s.bytes()
            n += 1
        if time.perf_counter() - t0 > seconds:
            break
    el = time.perf_counter() - t0
    return {"value": done_bytes / el / 1e9, "unit": "GB/s", "cores": nth, "kind": "port",
            "sample": f"{n} random instances of the uneven batch (conv_fft_par port, f32) in {el:.1f} s"}


# The benchmark's other single-instance cases, each through every variant
# that applies (device time of one call, CUDA-graph replay), with its
# normwise error against the f64 oracle: (key, description, x shape, kernel
# shape, mode, padding, dtype, variants)
VARIANT_CASES = [
    ("c1", "1-D f32 x[5000] * k[31], Full, Zeros", (5000,), (31,), "Full", "Zeros", "f32", ["direct", "bf16x3", "fft"]),
    ("c3", "3-D f32 x[10,100,200] * k[5,11,31], Same, Zeros", (10, 100, 200), (5, 11, 31), "Same", "Zeros", "f32",
     ["direct", "bf16x3", "fft"]),
    ("c3_complex", "3-D Complex<f32> x[10,100,200] * k[5,11,31] (re, im i.i.d. N(0,1)), Same, Zeros",
     (10, 100, 200), (5, 11, 31), "Same", "Zeros", "c32", ["direct", "bf16x3", "fft"]),
    ("2d_k31x31", "2-D f32 x[1024,1024] * k[31,31], Same, Zeros (a dense kernel of >= 15 taps per axis)",
     (1024, 1024), (31, 31), "Same", "Zeros", "f32", ["direct", "bf16x3", "fft"]),
]
VARIANT_ALGO = {"direct": 0, "bf16x3": 2, "fft": 1}


def measure_variants(reps=20):
    """Device time of one call of each variant on each VARIANT_CASES case
    (one call captured in a CUDA graph, replayed `reps` times between CUDA
    events), the FP32-equivalent rate 2 |y| taps / t, and the normwise error
    against the f64 oracle's direct loop."""
    out = {}
    for key, desc, xs, ksh, mode_n, pad_n, dt, variants in VARIANT_CASES:
        try:
            out[key] = _variant_case(desc, xs, ksh, mode_n, pad_n, dt, variants, reps)
        except Exception as ex:  # the line still prints; the case records why it has no figures
            out[key] = {"workload": desc, "error": f"{type(ex).__name__}: {ex}"[:200]}
    return out


def _variant_case(desc, xs, ksh, mode_n, pad_n, dt, variants, reps):
    import torch
    import ndconv
    from ndconv import _abi, build_problem, ConvMode, PaddingMode, with_dilation
    from oracle import oracle as O
    mode, pm = getattr(ConvMode, mode_n), getattr(PaddingMode, pad_n)
    rng = np.random.default_rng(3000 + len(xs))
    if dt == "c32":
        x = (rng.standard_normal(xs) + 1j * rng.standard_normal(xs)).astype(np.complex64)
        k = (rng.standard_normal(ksh) + 1j * rng.standard_normal(ksh)).astype(np.complex64)
        d64 = _abi.C64
    else:
        x = rng.random(xs, dtype=np.float32)
        k = rng.random(ksh, dtype=np.float32)
        d64 = _abi.F64
    st, y64 = O.conv(build_problem(d64, xs, with_dilation(k, 1), mode, pm),
                     x.astype(np.complex128 if dt == "c32" else np.float64),
                     k.astype(np.complex128 if dt == "c32" else np.float64))
    xd, kd = torch.from_numpy(x).cuda(), torch.from_numpy(k).cuda()
    res = {"workload": desc}
    for v in variants:
        algo = VARIANT_ALGO[v]
        for _ in range(3):
            y = ndconv.conv_algo(xd, kd, mode, pm, algo)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(g, stream=side):
                y = ndconv.conv_algo(xd, kd, mode, pm, algo)
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            g.replay()
        e1.record()
        torch.cuda.synchronize()
        us = e0.elapsed_time(e1) / reps * 1e3
        yh = y.cpu().numpy().astype(y64.dtype)
        err = float(np.linalg.norm(yh - y64) / np.linalg.norm(y64)) if st == 0 else None
        taps = float(np.prod(ksh))
        flops = (8.0 if dt == "c32" else 2.0) * float(np.prod(y64.shape)) * taps
        res[v] = {"us_per_call": us, "normwise_err": err, "fp32_equiv_tflops": flops / (us * 1e-6) / 1e12}
        del g
    fastest = min(variants, key=lambda v: res[v]["us_per_call"])
    res["fastest"] = fastest
    if "bf16x3" in variants:
        res["bf16x3_over_direct_speedup"] = res["direct"]["us_per_call"] / res["bf16x3"]["us_per_call"]
    return res


def measure_replicated(B=64, reps=10):
    """Configs 1 and 3 as B-fold replicated batches (distinct seeded
    instances, one submission per step) through the batched FFT, direct FP32
    and 3xBF16 tensor-core entry points: GB/s of algorithmic bytes and the
    f64-oracle error of instance 0."""
    import torch
    import ndconv
    from ndconv import _abi, build_problem, with_dilation, ConvMode, PaddingMode
    from oracle import oracle as O
    L = _abi.lib()
    cases = [("c1", "1-D f32 x[5000] * k[31], Full, Zeros", (5000,), (31,), ConvMode.Full),
             ("c3", "3-D f32 x[10,100,200] * k[5,11,31], Same, Zeros", (10, 100, 200), (5, 11, 31), ConvMode.Same)]
    out = {}
    for key, desc, xs_shape, ks_shape, mode in cases:
        pm = PaddingMode.Zeros
        rng = np.random.default_rng(5000 + len(xs_shape))
        xs_np = [rng.random(xs_shape, dtype=np.float32) for _ in range(B)]
        ks_np = [rng.random(ks_shape, dtype=np.float32) for _ in range(B)]
        xs = [torch.from_numpy(a).cuda() for a in xs_np]
        ks = [torch.from_numpy(a).cuda() for a in ks_np]
        p = build_problem(_abi.F32, xs_shape, with_dilation(ks[0], 1), mode, pm)
        p64 = build_problem(_abi.F64, xs_shape, with_dilation(ks_np[0], 1), mode, pm)
        st64, y64 = O.conv(p64, xs_np[0].astype(np.float64), ks_np[0].astype(np.float64))
        osh = (ctypes.c_int64 * 3)()
        assert L.ndconv_output_shape(ctypes.byref(p), 0, osh) == 0, _abi.last_error()
        oshape = tuple(osh[i] for i in range(len(xs_shape)))
        nbytes = 4 * (int(np.prod(xs_shape)) + int(np.prod(ks_shape)) + int(np.prod(oshape)))
        ys = [torch.empty(oshape, device="cuda") for _ in range(B)]
        PX, PK, PY = [torch.tensor([t.data_ptr() for t in ts], dtype=torch.int64, device="cuda") for ts in (xs, ks, ys)]
        sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        proc = ndconv.get_fft_processor(torch.float32)
        a = [ctypes.byref(p), B, ctypes.c_void_p(PX.data_ptr()), ctypes.c_void_p(PK.data_ptr()),
             ctypes.c_void_p(PY.data_ptr())]
        calls = {"fft": lambda: L.ndconv_conv_fft_batch(*a, proc._handle, sp),
                 "direct": lambda: L.ndconv_conv_batch(*a, sp),
                 "bf16x3": lambda: L.ndconv_conv_bf16x3_batch(*a, sp)}
        res = {"workload": f"{B} x {desc}, one batched submission per step", "bytes_per_instance": nbytes}
        for name, call in calls.items():
            try:
                for _ in range(3):
                    if call():
                        raise RuntimeError(_abi.last_error())
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    call()
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / reps
                y0 = ys[0].cpu().numpy().astype(np.float64)
                err = float(np.linalg.norm(y0 - y64) / np.linalg.norm(y64)) if st64 == 0 else None
                res[name] = {"gbs": nbytes * B / (ms * 1e-3) / 1e9, "ms_per_step": ms, "normwise_err": err}
            except Exception as ex:
                res[name] = {"error": f"{type(ex).__name__}: {ex}"[:200]}
        out[key] = res
    return out


def measure_c2_tensor(args, world, rank, local_rank, dist):
    """The headline's B instances through the batched 3xBF16 tensor-core
    direct path (ndconv_conv_bf16x3_batch, one persistent launch):
    device-resident time per step, the FP32-equivalent rate 2 |y| taps / t
    and the split-product bf16 rate (three products per tap) against the
    measured bf16 peak, and the f64-oracle error of instance 0."""
    import torch
    mode, pm, ndconv = problem_args()
    from ndconv import _abi, build_problem, with_dilation
    L = _abi.lib()
    B = args.batch
    xs_np, ks_np = c2_inputs(B, SEED_C2 + rank)
    xs = [torch.from_numpy(a).cuda() for a in xs_np]
    ks = [torch.from_numpy(a).cuda() for a in ks_np]
    p = build_problem(_abi.F32, SHAPE_X, with_dilation(ks[0], DIL), mode, pm)
    osh = (ctypes.c_int64 * 3)()
    assert L.ndconv_output_shape(ctypes.byref(p), 0, osh) == 0, _abi.last_error()
    out_shape = (osh[0], osh[1])
    ys = [torch.empty(out_shape, device="cuda") for _ in range(B)]
    P_X, P_K, P_Y = [torch.tensor([t.data_ptr() for t in ts], dtype=torch.int64, device="cuda") for ts in (xs, ks, ys)]
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def step():
        s = L.ndconv_conv_bf16x3_batch(ctypes.byref(p), B, ctypes.c_void_p(P_X.data_ptr()),
                                       ctypes.c_void_p(P_K.data_ptr()), ctypes.c_void_p(P_Y.data_ptr()), sp)
        if s:
            raise RuntimeError(_abi.last_error())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    from oracle import oracle as O
    p64 = build_problem(_abi.F64, SHAPE_X, with_dilation(ks_np[0], DIL), mode, pm)
    stt, y64 = O.conv(p64, xs_np[0].astype(np.float64), ks_np[0].astype(np.float64))
    err = float(np.linalg.norm(ys[0].cpu().numpy().astype(np.float64) - y64) / np.linalg.norm(y64)) if stt == 0 else None
    flops = 2.0 * float(np.prod(out_shape)) * float(np.prod(SHAPE_K)) * B
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            bf16_peak = float(json.load(f)["bf16_tflops"])
        peak_kind = "measured"
    except Exception:
        bf16_peak, peak_kind = 1900.0, "fallback"
    split_tflops = 3.0 * flops / (ms * 1e-3) / 1e12
    return {"workload": WORKLOAD_C2.format(B=B, what="conv on the tensor cores (3xBF16 split products)",
                                           form="batched (ndconv_conv_bf16x3_batch)"),
            "gbs": algorithmic_bytes(out_shape) * B * world / (ms * 1e-3) / 1e9, "ms_per_step": ms,
            "fp32_equiv_tflops": flops / (ms * 1e-3) / 1e12,
            "bf16_split_product_tflops": split_tflops,
            "bf16_peak_tflops": bf16_peak, "bf16_peak_source": f"MEASURED_PEAKS.json bf16_tflops ({peak_kind})",
            "useful_bf16_frac": split_tflops / bf16_peak,
            "normwise_err": err, "clocks": clk.summary()}


def measure_c2(args, algo, form, world, rank, local_rank, dist):
    """The 2-D case over B instances: conv_fft (algo 1) or conv (algo 0),
    batched or one call per instance; device-resident, plain per-instance
    and end-to-end (host-memory batch) timings, and the f64-oracle error of
    instance 0 (the i32 copy's bit-exactness for the direct path)."""
    import torch
    mode, pm, ndconv = problem_args()
    from ndconv import _abi, build_problem, with_dilation
    L = _abi.lib()
    B = args.batch
    xs_np, ks_np = c2_inputs(B, SEED_C2 + rank)
    xs = [torch.from_numpy(a).cuda() for a in xs_np]
    ks = [torch.from_numpy(a).cuda() for a in ks_np]
    p = build_problem(_abi.F32, SHAPE_X, with_dilation(ks[0], DIL), mode, pm)
    osh = (ctypes.c_int64 * 3)()
    st = L.ndconv_output_shape(ctypes.byref(p), algo, osh)
    assert st == 0, _abi.last_error()
    out_shape = (osh[0], osh[1])
    ys = [torch.empty(out_shape, device="cuda") for _ in range(B)]
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    proc = ndconv.get_fft_processor(torch.float32)
    pp = ctypes.byref(p)

    def ptrs(ts):
        return torch.tensor([t.data_ptr() for t in ts], dtype=torch.int64, device="cuda")

    def plain_step(xl, kl, yl):
        # the plain drop-in: one library call per instance
        for i in range(B):
            if algo == 1:
                s = L.ndconv_conv_fft(pp, ctypes.c_void_p(xl[i].data_ptr()), ctypes.c_void_p(kl[i].data_ptr()),
                                      ctypes.c_void_p(yl[i].data_ptr()), proc._handle, sp)
            else:
                s = L.ndconv_conv(pp, ctypes.c_void_p(xl[i].data_ptr()), ctypes.c_void_p(kl[i].data_ptr()),
                                  ctypes.c_void_p(yl[i].data_ptr()), sp)
            if s:
                raise RuntimeError(_abi.last_error())

    P_X, P_K, P_Y = ptrs(xs), ptrs(ks), ptrs(ys)

    def step():
        if form == "plain":
            return plain_step(xs, ks, ys)
        if algo == 1:
            s = L.ndconv_conv_fft_batch(pp, B, ctypes.c_void_p(P_X.data_ptr()), ctypes.c_void_p(P_K.data_ptr()),
                                        ctypes.c_void_p(P_Y.data_ptr()), proc._handle, sp)
        else:
            s = L.ndconv_conv_batch(pp, B, ctypes.c_void_p(P_X.data_ptr()), ctypes.c_void_p(P_K.data_ptr()),
                                    ctypes.c_void_p(P_Y.data_ptr()), sp)
        if s:
            raise RuntimeError(_abi.last_error())

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    # ---- device-resident timed region
    n0 = L.ndconv_kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        barrier()
    launches = L.ndconv_kernel_launches() - n0
    ms = e0.elapsed_time(e1) / args.steps
    plain_ms = None
    if form == "batched":
        plain_step(xs, ks, ys)
        barrier()
        e0.record(stream)
        for _ in range(max(1, args.steps // 2)):
            plain_step(xs, ks, ys)
        e1.record(stream)
        barrier()
        plain_ms = e0.elapsed_time(e1) / max(1, args.steps // 2)

    # ---- end to end: pinned host inputs, H2D + conv + D2H per step
    hx = [torch.from_numpy(a).pin_memory() for a in xs_np]
    hk = [torch.from_numpy(a).pin_memory() for a in ks_np]
    hy = [torch.empty(out_shape).pin_memory() for _ in range(B)]
    dx = [torch.empty_like(x) for x in xs]
    dk = [torch.empty_like(k) for k in ks]
    arr = ctypes.c_void_p * B
    HX, HK, HY = arr(*[t.data_ptr() for t in hx]), arr(*[t.data_ptr() for t in hk]), arr(*[t.data_ptr() for t in hy])

    def e2e_step():
        if form == "batched":
            # the library's host-memory batch: copies of one chunk overlap the
            # convolution of the previous one
            s = L.ndconv_conv_batch_host(pp, algo, B, HX, HK, HY, proc._handle if algo == 1 else None, sp)
            if s:
                raise RuntimeError(_abi.last_error())
            return
        for i in range(B):
            dx[i].copy_(hx[i], non_blocking=True)
            dk[i].copy_(hk[i], non_blocking=True)
        plain_step(dx, dk, ys)
        for i in range(B):
            hy[i].copy_(ys[i], non_blocking=True)

    for _ in range(2):
        e2e_step()
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    if dist:
        t = torch.tensor([ms, e2e_ms, plain_ms or 0.0], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, e2e_ms, pm_ = [float(v) for v in t.tolist()]
        plain_ms = pm_ if plain_ms is not None else None

    # ---- parity: instance 0 against the f64 oracle (its host-batch output too)
    from oracle import oracle as O
    p64 = build_problem(_abi.F64, SHAPE_X, with_dilation(ks_np[0], DIL), mode, pm)
    stt, y64 = O.conv(p64, xs_np[0].astype(np.float64), ks_np[0].astype(np.float64))
    err = None
    if stt == 0:
        err = max(float(np.linalg.norm(y.astype(np.float64) - y64) / np.linalg.norm(y64))
                  for y in (ys[0].cpu().numpy(), hy[0].numpy()))
    i32_exact = None
    if algo == 0:
        # the case's i32 copy (values Uniform{-100..100}): bit-exact against the oracle's direct loop
        xi, ki = c2_inputs(1, SEED_C2 + 7 + rank, np.int32)
        pi = build_problem(_abi.I32, SHAPE_X, with_dilation(ki[0], DIL), mode, pm)
        yi = ndconv.conv(torch.from_numpy(xi[0]).cuda(), with_dilation(torch.from_numpy(ki[0]).cuda(), DIL), mode, pm)
        sti, yio = O.conv(pi, xi[0], ki[0])
        i32_exact = bool(sti == 0 and np.array_equal(yi.cpu().numpy(), yio))
    return {"ms": ms, "plain_ms": plain_ms, "e2e_ms": e2e_ms, "err": err, "launches": int(launches),
            "clocks": clk.summary(), "out_shape": out_shape, "i32_exact": i32_exact,
            "h2d": int(4 * (np.prod(SHAPE_X) + np.prod(SHAPE_K)) * B), "d2h": int(4 * int(np.prod(out_shape)) * B)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--algo", default="fft", choices=["fft", "direct"])
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--form", default="batched", choices=["batched", "plain"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-seconds", type=float, default=0.0,
                    help="reference arm: stop after the step that passes this many seconds (0: run --steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="headline workload only (no direct and uneven-batch figures in config)")
    ap.add_argument("--config", default="c2", choices=["c2", "c4"])
    ap.add_argument("--n-instances", type=int, default=4096)
    ap.add_argument("--dispatch", default="mlp", choices=["mlp", "model"])
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        import __graft_entry__  # noqa: F401  (paths)
        from oracle import oracle as O
        O.build()
        return run_reference(args, rank, world)

    import torch
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    try:
        if args.config == "c4":
            return bench_uneven(args, world, rank, local_rank, dist)
        algo = 1 if args.algo == "fft" else 0
        r = measure_c2(args, algo, args.form, world, rank, local_rank, dist)
        extra_direct = extra_uneven = extra_variants = extra_tensor = extra_replicated = None
        if not args.no_extra and algo == 1 and args.form == "batched":
            extra_direct = measure_c2(args, 0, "batched", world, rank, local_rank, dist)
            try:
                extra_tensor = measure_c2_tensor(args, world, rank, local_rank, dist)
            except Exception as ex:  # the line still prints; the block says why it has no figures
                extra_tensor = {"error": f"{type(ex).__name__}: {ex}"[:200]}
            extra_uneven = measure_uneven(args, world, rank, local_rank, dist)
            if rank == 0:
                extra_variants = measure_variants()
                try:
                    extra_replicated = measure_replicated()
                except Exception as ex:  # the line still prints; the block says why it has no figures
                    extra_replicated = {"error": f"{type(ex).__name__}: {ex}"[:200]}
        if rank != 0:
            return
        B = args.batch
        out_shape = r["out_shape"]
        bytes_inst = algorithmic_bytes(out_shape)

        def gbs(ms):
            return bytes_inst * B * world / (ms * 1e-3) / 1e9

        peak, peak_kind = peaks()
        achieved = bytes_inst / (r["ms"] / B * 1e-3) / 1e9  # one instance's convolution
        cpu = None
        if not args.no_cpu_baseline and world == 1 and algo == 1:  # host-core baseline at N = 1 only
            cpu = cpu_baseline(args.cpu_seconds, B)
        traffic = PROFILED_TRAFFIC.get(args.algo) if args.form == "batched" else None
        config = {"workload": WORKLOAD_C2.format(B=B, what="conv_fft" if algo else "conv", form=args.form),
                  "metric_detail": METRIC_DETAIL, "batch_per_gpu": B, "algo": args.algo, "form": args.form,
                  "plain_per_instance_gbs": gbs(r["plain_ms"]) if r["plain_ms"] else None,
                  "batched_over_plain": (r["plain_ms"] / r["ms"]) if r["plain_ms"] else None,
                  "l2": "inputs (256 MB per GPU) larger than L2, no flush"}
        if extra_direct:
            d = extra_direct
            fma = fp32_fma_roofline(out_shape, d["ms"] / B, d["clocks"].get("sm_mhz"))
            config["direct"] = {"workload": WORKLOAD_C2.format(B=B, what="conv (direct FP32)", form="batched"),
                                "gbs": gbs(d["ms"]), "ms_per_step": d["ms"],
                                "plain_per_instance_gbs": gbs(d["plain_ms"]),
                                "batched_over_plain": d["plain_ms"] / d["ms"], "e2e_gbs": gbs(d["e2e_ms"]),
                                "fp32_tflops": fma["achieved"], "fp32_fma_peak_tflops": fma["peak"],
                                "fp32_fma_frac": fma["frac"], "normwise_err": d["err"],
                                "i32_bit_exact": d["i32_exact"], "gpu_launches": d["launches"],
                                "clocks": d["clocks"]}
        if extra_uneven:
            config["uneven_batch"] = uneven_summary(extra_uneven, world)
        if extra_variants:
            config["variants"] = extra_variants
        if extra_tensor:
            config["direct_tensor_cores"] = extra_tensor
        if extra_replicated:
            config["replicated"] = extra_replicated
        line = {
            "metric": METRIC,
            "value": gbs(r["ms"]), "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32",
            "data": f"synthetic (seeded Uniform[0,1), distinct data and kernel per instance, seed {SEED_C2} + rank)",
            "config": config,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": PROFILED_TRAFFIC_SOURCE if traffic else None,
                         "kernel": "one instance's convolution (all its launches)",
                         "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
            "cpu_baseline": cpu,
            "e2e": {"value": gbs(r["e2e_ms"]), "unit": "GB/s", "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": r["d2h"]},
            "gpu_launches": r["launches"],
            "clocks": r["clocks"],
            "normwise_err_vs_f64": r["err"],
        }
        if not algo:
            # the direct path is bound by the FP32 FMA rate, not by HBM
            line["compute_roofline"] = fp32_fma_roofline(out_shape, r["ms"] / B, r["clocks"].get("sm_mhz"))
            line["i32_bit_exact"] = r["i32_exact"]
        print(json.dumps(line), flush=True)
    finally:
        if dist:
            dist.barrier()
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
