"""Builds and runs the reference-style C++ test against the C++20 header."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_test(ttg, tmp_path):
    libdir = os.path.dirname(ttg.library_path())
    exe = str(tmp_path / "test_header_round")
    subprocess.check_call(["g++", "-std=c++20", "-O2", "-Wall", "-Wextra",
                           "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "test_header_round.cpp"),
                           "-L", libdir, "-lttgpu", f"-Wl,-rpath,{libdir}", "-o", exe])
    return exe


def test_header_compiles(ttg, tmp_path):
    assert os.path.exists(build_test(ttg, tmp_path))


@pytest.mark.gpu
def test_header_round_runs(ttg, tmp_path):
    exe = build_test(ttg, tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "OK" in out.stdout
