"""The JSON line of bench.py's reference arm (runs on the CPU: the oracle
port on all host threads) carries the contract's keys."""
import argparse
import json


def test_reference_arm_line(capsys, monkeypatch):
    import bench
    monkeypatch.delenv("RANK", raising=False)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    bench.run_reference(argparse.Namespace(gpus=1, steps=1, warmup=0, count=4096))
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0.0 and line["n_gpus"] == 1
    assert "workload" in line["config"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert e2e["unit"] == line["unit"]


def test_roofline_objects(tmp_path):
    import bench
    hbm, bf16, src = bench.measured_peaks()
    assert hbm > 0 and bf16 > 0
    r = bench.roofline_tensor(6.5e11, 1000.0, 1.25, traffic=6e10)
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s" and r["peak"] == bf16
    assert abs(r["achieved"] - 0.65) < 1e-12 and abs(r["frac"] - 0.65 / bf16) < 1e-15
    assert abs(r["fp64_pipe"]["frac"] - 0.52) < 1e-12 and r["traffic"] == 6e10
    # without the measured-peaks file: the published fallback, and it says so
    hbm2, bf2, src2 = bench.measured_peaks(str(tmp_path / "absent.json"))
    assert (hbm2, bf2) == (6800.0, 1900.0) and "fallback" in src2


def test_reference_arm_loads_only_the_oracle():
    # The reference arm must not map the product library: it builds its
    # inputs with the oracle's own generator and rounds them with the oracle.
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import argparse, sys, bench\n"
            "bench.run_reference(argparse.Namespace(gpus=1, steps=1, warmup=0, count=4096))\n"
            "assert 'tensor_train_gb300' not in sys.modules, 'product package imported'\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert 'libttgpu' not in maps, 'product library mapped'\n")
    env = dict(os.environ)
    env.pop("RANK", None)
    env.pop("WORLD_SIZE", None)
    r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    import json
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
