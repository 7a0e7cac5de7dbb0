"""The backend for the reference's factory seam (include/genfft/gb300_backend.h)
compiles and links, without a GPU:
  * against the reference's own headers (a genFFT checkout named by
    GENFFT_REFERENCE_DIR; skipped when it is not set): the reference's
    classes with genfft::gb300::GetImpl / GetVertImpl / GetDITImpl;
  * against the interface declaration with the reference's signatures
    (include/genfft/backend_iface.h) and the drop-in header, whose classes
    take the reference's factory template parameters."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = "/usr/local/cuda"


@pytest.fixture(scope="module")
def lib_dir():
    from genfft_gb300 import build
    return os.path.dirname(build.build())


def compile_cpp(src, exe, lib_dir, extra_inc=()):
    cmd = ["g++", "-O1", "-std=c++17", *[f"-I{d}" for d in extra_inc], f"-I{ROOT}/include", f"-I{CUDA}/include",
           os.path.join(ROOT, "tests", "cpp", src), "-o", exe, f"-L{lib_dir}", "-lgenfft_gb300",
           f"-L{CUDA}/lib64", "-lcudart", f"-Wl,-rpath,{lib_dir}"]
    return subprocess.run(cmd, capture_output=True, text=True)


def test_seam_against_interface_declaration(lib_dir, tmp_path):
    r = compile_cpp("seam_test.cpp", str(tmp_path / "seam_test"), lib_dir)
    assert r.returncode == 0, r.stderr[-3000:]


def test_shim_test_cases_compile(lib_dir, tmp_path):
    r = compile_cpp("shim_test.cpp", str(tmp_path / "shim_test"), lib_dir)
    assert r.returncode == 0, r.stderr[-3000:]


def test_reference_classes_take_gb300_factories(lib_dir, tmp_path):
    ref = os.environ.get("GENFFT_REFERENCE_DIR", "")
    inc = os.path.join(ref, "include")
    if not ref or not os.path.isdir(os.path.join(inc, "genFFT")):
        pytest.skip("no genFFT checkout named by GENFFT_REFERENCE_DIR")
    r = compile_cpp("seam_ref_test.cpp", str(tmp_path / "seam_ref_test"), lib_dir, extra_inc=(inc,))
    assert r.returncode == 0, r.stderr[-3000:]
