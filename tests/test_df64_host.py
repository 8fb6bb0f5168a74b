"""Builds and runs tests/cpp/test_df64_host.cpp on the CPU: the bit-level
FP64 <-> double-float conversions, the double-float reciprocal and square
root, and the GEMM tiles' live-row rule, from the kernels' own headers
(host code of an nvcc build; nothing runs on a GPU)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_df64_arithmetic_on_host(tmp_path):
    nvcc = next((c for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc"))
                 if c and os.path.exists(c)), None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "test_df64_host")
    subprocess.check_call([nvcc, "-std=c++17", "-O2", "-x", "cu",
                           "-gencode", "arch=compute_103a,code=sm_103a",
                           "-I", os.path.join(ROOT, "tensor_train_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "cpp", "test_df64_host.cpp"), "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "OK" in out.stdout
