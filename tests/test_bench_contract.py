"""The benchmark's reference arm on CPU: one JSON line with the contract's keys,
the same workload description as the GPU arm, and a time-like metric. The
oracle port runs on a tiny sample so the test takes a second or two."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bench_kind() -> str:
    sys.path.insert(0, ROOT)
    import bench

    return bench.cpu_kind()


def test_reference_arm_json_line():
    out = subprocess.run(
        [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2", "--warmup", "1",
         "--cpu-sample-n2", "64", "--n2", "8192"],
        capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["higher_is_better"] is False and d["unit"] == "ms" and d["value"] > 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == bench_kind() and d["cpu_baseline"]["cores"] >= 1
    # a scaled sample says so, with the sample and the factor
    cb = d["cpu_baseline"]
    assert cb["extrapolated"] is True and cb["sample_n2"] == 64 and cb["scale_n3"] == (8192 / 64) ** 3
    assert cb["fits_in_driver_run"] is False
    assert cb["reference_measured_directly"]["n2"] == 8192

    sys.path.insert(0, ROOT)
    import bench

    assert d["config"] == bench.workload_config(8192, 1)
    assert d["metric"] == bench.METRIC


def test_cpu_baseline_falls_back_to_the_port(monkeypatch):
    """Where the compiled reference does not exist or does not load (the GPU
    host has neither its sources nor x86 binaries), the baseline is the port
    on an n2 = 1024 sample."""
    sys.path.insert(0, ROOT)
    import bench
    from oracle import ref

    monkeypatch.setattr(ref, "available", lambda: False)
    assert bench.cpu_kind() == "port"
    assert bench.cpu_sample_n2(0) == 1024
    assert bench.cpu_sample_n2(512) == 512
    ms, raw = bench.cpu_sample(64, 128, 1)
    assert raw > 0 and abs(ms - raw * 1e3 * 8) < 1e-6 * ms
