"""CPU check of bench.py's reference arm: one bounded run of the CPU port of
conv_fft_par prints one JSON line with the keys every bench line carries, the
same metric and workload as the GPU arm, and an e2e figure with no
host-device bytes; both arms draw the same seeded instances."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "1", "--batch", "2"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    sys.path[:0] = [ROOT]
    import bench
    assert d["metric"] == bench.METRIC
    assert d["impl"] == "reference" and d["unit"] == "GB/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert "workload" in d["config"]
    # the GPU arm's headline line names the same workload for the same batch
    assert d["config"]["workload"] == bench.WORKLOAD_C2.format(B=2, what="conv_fft", form="batched")
    assert d["config"]["batch_per_gpu"] == 2


def test_both_arms_draw_the_same_instances():
    sys.path[:0] = [ROOT]
    import numpy as np
    import bench
    a = bench.c2_inputs(3, bench.SEED_C2)
    b = bench.c2_inputs(3, bench.SEED_C2)
    for u, v in zip(a[0] + a[1], b[0] + b[1]):
        assert np.array_equal(u, v)
    assert not np.array_equal(a[0][0], a[0][1])  # distinct instances
