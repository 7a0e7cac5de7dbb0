"""The drop-in C++ header (include/genfft/fft.h) compiled against the
reference's own test cases (tests/cpp/shim_test.cpp) and run on the GPU."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_shim(gfft, tmp_path):
    lib_dir = os.path.dirname(gfft.lib_path())
    exe = str(tmp_path / "shim_test")
    cuda = "/usr/local/cuda"
    cmd = ["g++", "-O2", "-std=c++17", f"-I{ROOT}/include", f"-I{cuda}/include",
           os.path.join(ROOT, "tests", "cpp", "shim_test.cpp"), "-o", exe,
           f"-L{lib_dir}", "-lgenfft_gb300", f"-L{cuda}/lib64", "-lcudart",
           f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{cuda}/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-2000:])
    assert "OK: 0 failures" in r.stdout
