"""Benchmark: convolution GB/s and % of HBM roofline on one GB300.

Workload (the reference's 2-D benchmark case, batched): B
independent instances of a 2-D f32 convolution x[200, 5000] with a kernel
[11, 31] dilated by 2, ConvMode::Same, PaddingMode::Custom([Reflect,
Circular]); every instance has its own seeded Uniform[0,1) data and kernel.
A step is one pass of conv_fft (default) or conv over all B instances.
B = 64 makes the inputs (256 MB) larger than L2, so no flush is needed.

Metric: algorithmic bytes 4 * (|x| + |k| + |y|) per instance / time.
  value   device-resident inputs, CUDA-event timed (max over ranks)
  e2e     the same calls with pinned-host inputs: H2D copy + conv + D2H of
          the outputs inside the timed region
Reference arm (--impl reference): the oracle port of conv_fft_par (same
algorithm as the crate, rayon-style threads on all host cores) on a
bounded sample of the same workload.
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

# DRAM bytes per instance of the batched FFT path from one ncu capture (one
# wave of 16 instances, caches flushed between the two launches): an upper bound
PROFILED_TRAFFIC = {"fft": 12.27e6}

# the benchmark's metric; every line (both arms, both workloads) reports it
METRIC = "conv GB/s & % HBM roofline, batched+tuned vs plain GPU, err ≤1e-5 vs FP64"
METRIC_DETAIL = "GB/s of algorithmic bytes 4*(|x|+|k|+|y|) per instance"

SHAPE_X = (200, 5000)
SHAPE_K = (11, 31)
DIL = 2


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


def cpu_baseline(seconds=10.0, nthreads=None, algo="fft"):
    """The oracle port on the host cores, one instance per call, repeated for
    ~`seconds`: conv_fft_par on all cores for the FFT line, the crate's
    single-threaded direct loop (ConvExt::conv) for the direct line.
    Returns (GB/s, cores, sample text)."""
    from oracle import oracle as O
    from ndconv import _abi, build_problem, with_dilation
    mode, pm, _ = problem_args()
    direct = algo == "direct"
    nthreads = 1 if direct else (nthreads or os.cpu_count() or 1)
    rng = np.random.default_rng(12345)
    x = rng.random(SHAPE_X).astype(np.float32)
    k = rng.random(SHAPE_K).astype(np.float32)
    p = build_problem(_abi.F32, SHAPE_X, with_dilation(k, DIL), mode, pm)

    def once():
        return O.conv(p, x, k) if direct else O.conv_fft(p, x, k, nthreads)

    st, y = once()  # warm-up
    assert st == 0
    n, t0 = 0, time.perf_counter()
    while True:
        once()
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    gbs = algorithmic_bytes(y.shape) * n / el / 1e9
    what = "conv port, direct loop, 1 thread" if direct else "conv_fft_par port"
    return gbs, nthreads, f"{n} instances of x[200,5000]*k[11,31] ({what}, f32) in {el:.1f} s"


def run_reference(args, rank, world):
    if rank != 0:
        return
    steps, warm = args.steps, args.warmup
    # each step: a bounded sample (--ref-instances instances) of the workload
    from oracle import oracle as O
    from ndconv import _abi, build_problem, with_dilation
    mode, pm, _ = problem_args()
    nth = os.cpu_count() or 1
    rng = np.random.default_rng(12345)
    x = rng.random(SHAPE_X).astype(np.float32)
    k = rng.random(SHAPE_K).astype(np.float32)
    p = build_problem(_abi.F32, SHAPE_X, with_dilation(k, DIL), mode, pm)
    for _ in range(max(1, warm)):
        st, y = O.conv_fft(p, x, k, nth)
    per_step = max(1, int(args.ref_instances))
    t0 = time.perf_counter()
    for _ in range(steps):
        for _ in range(per_step):
            O.conv_fft(p, x, k, nth)
    el = time.perf_counter() - t0
    gbs = algorithmic_bytes(y.shape) * per_step * steps / el / 1e9
    sample = f"{per_step} instance(s) of x[200,5000]*k[11,31] per step (conv_fft_par port, f32)"
    line = {"metric": METRIC,
            "value": gbs, "unit": "GB/s", "n_gpus": world, "steps": steps, "warmup": warm,
            "ms_per_step": el / steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Uniform[0,1))",
            "impl": "reference",
            "config": {"workload": "2-D f32 x[200,5000] * k[11,31] dilation 2, Same, "
                                   "Custom([Reflect, Circular]); conv_fft",
                       "metric_detail": METRIC_DETAIL},
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


def bench_uneven(args, world, rank, local_rank):
    """The uneven batch: independent instances in one persistent
    launch (device work queue, CUDA graph), against the same instances
    through the per-instance entry points (the plain drop-in)."""
    import torch
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
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
        avail = default_available()
        avail[1] = 0.0  # the tensor-core variant is not a persistent-queue task
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
    peak, peak_kind = peaks()
    value = bytes_step * world / (ms * 1e-3) / 1e9
    # parity spot checks against the f64 oracle (largest direct and FFT instances that stay cheap)
    from oracle import oracle as O
    from ndconv import build_problem
    errs = []
    for want in (0, 1):
        cand = [i for i, s in enumerate(specs) if (algos[i] != 0) == bool(want)]
        cand.sort(key=lambda i: specs[i].out_shape()[0] * 0 + int(np.prod(specs[i].out_shape())) *
                  int(np.prod(specs[i].kshape)))
        for i in cand[len(cand) // 2: len(cand) // 2 + 2]:
            s = specs[i]
            x0, k0 = xs[i].cpu().numpy().astype(np.float64), ks[i].cpu().numpy().astype(np.float64)
            p = build_problem(_abi.F64, s.shape, with_dilation(k0, s.dilation), s.conv_mode(), s.padding_mode())
            st, y64 = O.conv(p, x0, k0)
            if st == 0:
                y = ys[i].cpu().numpy().astype(np.float64)
                errs.append(float(np.linalg.norm(y - y64) / max(np.linalg.norm(y64), 1e-300)))
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline and world == 1:  # host-core baseline at N = 1 only
            cpu = cpu_baseline_uneven(specs, args.cpu_seconds)
        line = {
            "metric": METRIC,
            "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded; uneven-batch distribution)",
            "config": {"workload": f"uneven batch: {len(specs)} instances (rank 1/2/3 = 60/35/5%, "
                                   "2^8..2^20 elements, odd kernels 3..127, dilation/stride 1|2, "
                                   "Zeros/Reflect/Replicate/Circular), one persistent launch + CUDA graph",
                       "metric_detail": METRIC_DETAIL,
                       "instances_per_gpu": len(specs), "algos": {"direct": int(sum(a == 0 for a in algos)),
                                                                  "fft": int(sum(a != 0 for a in algos))},
                       "dispatcher": {"mlp": "trained network (ndconv/data/dispatcher_mlp.json)",
                                      "model": "cost model"}[args.dispatch], "plan": info,
                       "plain_per_instance_gbs": bytes_step * world / (plain_ms * 1e-3) / 1e9,
                       "batched_over_plain": plain_ms / ms,
                       "plain_dropin_gbs": bytes_step * world / (dropin_ms * 1e-3) / 1e9,
                       "batched_tuned_over_plain_dropin": dropin_ms / ms,
                       "plain_note": "plain = per-instance calls with the same picks; plain drop-in = "
                                     "per-instance calls with the library's default (cost model) picks",
                       "l2": f"inputs {xbuf.numel() * 4 / 1e9:.2f} GB per GPU, larger than L2, no flush"},
            "roofline": {"bound": "hbm", "achieved": bytes_step / (ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": bytes_step / (ms * 1e-3) / 1e9 / peak, "traffic": None,
                         "kernel": "persistent batch kernel (one launch per step, plus standalone launches)",
                         "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
            "cpu_baseline": cpu,
            "e2e": {"value": bytes_step * world / (e2e_ms * 1e-3) / 1e9, "unit": "GB/s",
                    "h2d_bytes_per_step": int((xbuf.numel() + kbuf.numel()) * 4),
                    "d2h_bytes_per_step": int(ybuf.numel() * 4)},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "normwise_err_vs_f64": max(errs) if errs else None,
        }
        print(json.dumps(line), flush=True)
    plan.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


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
    ap.add_argument("--ref-instances", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
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

    if args.config == "c4":
        return bench_uneven(args, world, rank, local_rank)
    import torch
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    mode, pm, ndconv = problem_args()
    from ndconv import _abi, build_problem, with_dilation
    L = _abi.lib()

    B = args.batch
    gen = torch.Generator(device="cuda").manual_seed(1000 + rank)
    xs = [torch.rand(SHAPE_X, generator=gen, device="cuda") for _ in range(B)]
    ks = [torch.rand(SHAPE_K, generator=gen, device="cuda") for _ in range(B)]
    p = build_problem(_abi.F32, SHAPE_X, with_dilation(ks[0], DIL), mode, pm)
    osh = (ctypes.c_int64 * 3)()
    algo = 1 if args.algo == "fft" else 0
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

    def batched_step_ptrs(px, pk, py):
        if algo == 1:
            s = L.ndconv_conv_fft_batch(pp, B, ctypes.c_void_p(px.data_ptr()), ctypes.c_void_p(pk.data_ptr()),
                                        ctypes.c_void_p(py.data_ptr()), proc._handle, sp)
        else:
            s = L.ndconv_conv_batch(pp, B, ctypes.c_void_p(px.data_ptr()), ctypes.c_void_p(pk.data_ptr()),
                                    ctypes.c_void_p(py.data_ptr()), sp)
        if s:
            raise RuntimeError(_abi.last_error())

    P_X, P_K, P_Y = ptrs(xs), ptrs(ks), ptrs(ys)

    def step(xl, kl, yl):
        if args.form == "plain":
            return plain_step(xl, kl, yl)
        if xl is xs:
            return batched_step_ptrs(P_X, P_K, P_Y)
        return batched_step_ptrs(ptrs(xl), ptrs(kl), ptrs(yl))

    for _ in range(args.warmup):
        step(xs, ks, ys)
    torch.cuda.synchronize()

    # ---- device-resident timed region
    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    barrier()
    n0 = L.ndconv_kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step(xs, ks, ys)
        e1.record(stream)
        barrier()
    launches = L.ndconv_kernel_launches() - n0
    ms = e0.elapsed_time(e1) / args.steps
    plain_ms = None
    if args.form == "batched":
        plain_step(xs, ks, ys)
        barrier()
        e0.record(stream)
        for _ in range(max(1, args.steps // 2)):
            plain_step(xs, ks, ys)
        e1.record(stream)
        barrier()
        plain_ms = e0.elapsed_time(e1) / max(1, args.steps // 2)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    bytes_step = algorithmic_bytes(out_shape) * B
    value = bytes_step * world / (ms * 1e-3) / 1e9
    per_launch_ms = ms / B  # one instance's convolution
    peak, peak_kind = peaks()
    achieved = algorithmic_bytes(out_shape) / (per_launch_ms * 1e-3) / 1e9

    # ---- end to end: pinned host inputs, H2D + conv + D2H per step
    hx = [x.cpu().pin_memory() for x in xs]
    hk = [k.cpu().pin_memory() for k in ks]
    hy = [torch.empty(out_shape).pin_memory() for _ in range(B)]
    dx = [torch.empty_like(x) for x in xs]
    dk = [torch.empty_like(k) for k in ks]

    PD_X, PD_K = ptrs(dx), ptrs(dk)
    arr = ctypes.c_void_p * B
    HX, HK, HY = arr(*[t.data_ptr() for t in hx]), arr(*[t.data_ptr() for t in hk]), arr(*[t.data_ptr() for t in hy])

    def e2e_step():
        if args.form == "batched":
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
        t = torch.tensor([e2e_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    h2d = 4 * (np.prod(SHAPE_X) + np.prod(SHAPE_K)) * B
    d2h = 4 * int(np.prod(out_shape)) * B

    # ---- parity spot check on instance 0 against the f64 oracle
    from oracle import oracle as O
    x0, k0 = xs[0].cpu().numpy(), ks[0].cpu().numpy()
    p64 = build_problem(_abi.F64, SHAPE_X, with_dilation(k0, DIL), mode, pm)
    stt, y64 = O.conv(p64, x0.astype(np.float64), k0.astype(np.float64))
    y0 = ys[0].cpu().numpy().astype(np.float64)
    err = float(np.linalg.norm(y0 - y64) / np.linalg.norm(y64)) if stt == 0 else None

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline and world == 1:  # host-core baseline at N = 1 only
            gbs, cores, sample = cpu_baseline(args.cpu_seconds, algo=args.algo)
            cpu = {"value": gbs, "unit": "GB/s", "cores": cores, "kind": "port", "sample": sample}
        line = {
            "metric": METRIC,
            "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded Uniform[0,1), distinct data and kernel per instance)",
            "config": {"workload": f"{B} x 2-D f32 x[200,5000] * k[11,31] dilation 2, Same, "
                                   f"Custom([Reflect, Circular]); {'conv_fft' if algo else 'conv'}, "
                                   f"{args.form} submission",
                       "metric_detail": METRIC_DETAIL,
                       "batch_per_gpu": B, "algo": args.algo, "form": args.form,
                       "plain_per_instance_gbs": (bytes_step * world / (plain_ms * 1e-3) / 1e9) if plain_ms else None,
                       "batched_over_plain": (plain_ms / ms) if plain_ms else None,
                       "l2": "inputs (256 MB per GPU) larger than L2, no flush"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": PROFILED_TRAFFIC.get(args.algo) if args.form == "batched" else None,
                         "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per instance, "
                                            "profiles/conv_fft_rowspectral_kernels_full.md")
                         if args.algo == "fft" and args.form == "batched" else None,
                         "kernel": "one instance's convolution (all its launches)",
                         "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
            "cpu_baseline": cpu,
            "e2e": {"value": bytes_step * world / (e2e_ms * 1e-3) / 1e9, "unit": "GB/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "normwise_err_vs_f64": err,
        }
        if not algo:
            # the direct path is bound by the FP32 FMA rate, not by HBM
            line["compute_roofline"] = fp32_fma_roofline(out_shape, per_launch_ms, line["clocks"].get("sm_mhz"))
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
