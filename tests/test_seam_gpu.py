"""The GB300 backend objects of the reference's factory seam
(genfft/gb300_backend.h: GetImpl, GetVertImpl, GetDITImpl) driven through
the interface declared with the reference's signatures, and the drop-in
class with a factory named explicitly, checked against the golden vectors
the reference itself produced (tests/golden)."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = "/usr/local/cuda"


@pytest.fixture(scope="module")
def exe(gfft, tmp_path_factory):
    lib_dir = os.path.dirname(gfft.lib_path())
    out = str(tmp_path_factory.mktemp("seam") / "seam_test")
    cmd = ["g++", "-O2", "-std=c++17", f"-I{ROOT}/include", f"-I{CUDA}/include",
           os.path.join(ROOT, "tests", "cpp", "seam_test.cpp"), "-o", out, f"-L{lib_dir}", "-lgenfft_gb300",
           f"-L{CUDA}/lib64", "-lcudart", f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{CUDA}/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def call(exe, tmp_path, op, x, n, cols=0):
    dt = np.complex64 if x.dtype in (np.complex64, np.float32) else np.complex128
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    np.ascontiguousarray(x, dtype=dt).tofile(fin)
    r = subprocess.run([exe, op, "f" if dt == np.complex64 else "d", str(n), str(cols), fin, fout],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (op, n, r.returncode, r.stderr[-2000:])
    return np.fromfile(fout, dtype=dt)


def close(a, b, eps):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return a.shape == b.shape and np.max(np.abs(a.real - b.real), initial=0) <= eps and \
        np.max(np.abs(a.imag - b.imag), initial=0) <= eps


def bitrev(n):
    bits = n.bit_length() - 1
    return np.array([int(format(i, f"0{bits}b")[::-1], 2) if bits else 0 for i in range(n)])


def test_get_impl_no_scramble_golden(exe, golden, oracle, tmp_path):
    # FFTBase::forward: in place, the input read as bit-reversed (FFTLevel.h:43-59)
    o = oracle.Impl("oracle")
    seen = 0
    for k in sorted({f.rsplit("/", 1)[0] for f in golden.files if f.startswith("c2c_f32_")}):
        if k + "/noscr_fwd_generic" not in golden.files:
            continue
        x = golden[k + "/in"]
        n = x.size
        eps = oracle.fft_eps(x.dtype, n) * 1.5
        assert close(call(exe, tmp_path, "fft_fwd", x, n), golden[k + "/noscr_fwd_generic"], eps), k
        assert close(call(exe, tmp_path, "fft_inv", x, n), o.fft_no_scramble(x, True), eps), k
        seen += 1
    assert seen >= 8


def test_get_impl_double(exe, oracle, tmp_path):
    o = oracle.Impl("oracle")
    rng = np.random.default_rng(5)
    for n in (1, 8, 512, 8192, 1 << 16):
        x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex128)
        assert close(call(exe, tmp_path, "fft_fwd", x, n), o.fft_no_scramble(x, False),
                     oracle.fft_eps(x.dtype, n) * 1.5), n


def test_get_vert_impl_golden(exe, golden, oracle, tmp_path):
    # FFTVertBase::forward: rows bit-reversed on input (FFTVert::transform
    # scrambles them first, fft.h:145-150), stride in scalars
    for k in sorted({f.rsplit("/", 1)[0] for f in golden.files if f.startswith("vert_")}):
        x = golden[k + "/in"]
        n, cols = x.shape
        xs = x[bitrev(n)]
        eps = oracle.fft_eps(x.dtype, n) * 1.5
        assert close(call(exe, tmp_path, "vert_fwd", xs, n, cols), golden[k + "/fwd_generic"], eps), k
        assert close(call(exe, tmp_path, "vert_inv", xs, n, cols), golden[k + "/inv_generic"], eps), k


def test_get_dit_impl_golden(exe, golden, oracle, tmp_path):
    for k in sorted({f.rsplit("/", 1)[0] for f in golden.files if f.startswith("dit_f32_")}):
        z = golden[k + "/in"]
        n = 2 * z.size
        eps = oracle.fft_eps(z.dtype, n) * 1.5
        # the golden buffer holds the reference's n-element output; half
        # mode writes its first n/2+1 bins
        assert close(call(exe, tmp_path, "dit_half", z, n), golden[k + "/half_generic"][:n // 2 + 1], eps), k
        assert close(call(exe, tmp_path, "dit_full", z, n), golden[k + "/full_generic"], eps), k


def test_classes_with_named_factories(exe, golden, oracle, tmp_path):
    # genfft::FFT<T, gb300::GetImpl> (the C-ABI path) and genfft::FFT<T, f>
    # with a CPU backend f (the reference's host algorithm through f)
    for n in (1, 2, 16, 256, 1024):
        k = f"c2c_f32_{n}"
        x = golden[k + "/in"]
        eps = oracle.fft_eps(x.dtype, n) * 1.5
        assert close(call(exe, tmp_path, "cls_fwd", x, n), golden[k + "/fwd_generic"], eps), k
        if n <= 256:
            assert close(call(exe, tmp_path, "cls_custom", x, n), golden[k + "/fwd_generic"], eps), k
