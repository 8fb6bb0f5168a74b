"""include/ttg.h from plain C11 (-pedantic -Werror), linked against the
library: the calls a cgo / JNI / ctypes binding makes, up to the point where
device work would start."""
import os
import subprocess


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_header_and_argument_checks(ttg, tmp_path):
    libdir = os.path.dirname(ttg.library_path())
    exe = str(tmp_path / "test_c_abi")
    subprocess.check_call(["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-pedantic", "-Werror",
                           "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "c", "test_c_abi.c"),
                           "-L", libdir, "-lttgpu", f"-Wl,-rpath,{libdir}", "-lm", "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "test_c_abi: OK" in out.stdout
