"""The C-ABI library loads without a GPU and exports every entry point the
public headers declare; argument validation answers before any CUDA call."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b(gfft_[a-z0-9_]+)\s*\(", src):
            syms.add(m.group(1))
    return syms


@pytest.fixture(scope="module")
def L():
    import genfft_gb300 as G
    from genfft_gb300 import build
    build.build()
    return G.lib()


def test_every_declared_symbol_is_exported(L):
    syms = declared_symbols()
    assert len(syms) >= 10
    for s in sorted(syms):
        assert hasattr(L, s), f"{s} declared in include/ but not exported"


def test_python_binding_covers_header():
    import genfft_gb300 as G
    assert declared_symbols() <= set(G.SIGNATURES), declared_symbols() - set(G.SIGNATURES)


def test_version_and_strings(L):
    assert L.gfft_version() == 1
    assert L.gfft_status_string(0) == b"success"
    assert L.gfft_status_string(1) == b"invalid size"
    assert L.gfft_max_fused_size(0) == 1 << 14
    assert L.gfft_max_fused_size(1) == 1 << 13
    assert L.gfft_max_fused_size(7) == 0


@pytest.mark.parametrize("n0,batch,dtype,mode,flags,status", [
    (3, 1, 0, 0, 0, 1),        # not a power of two
    (0, 1, 0, 0, 0, 1),        # zero size
    (-4, 1, 0, 0, 0, 1),       # negative
    (64, 0, 0, 0, 0, 1),       # empty batch
    (64, 1, 5, 0, 0, 2),       # bad dtype
    (64, 1, 0, 9, 0, 2),       # bad mode
    (64, 1, 0, 0, 0x80, 2),    # unknown flag
    (1024, 1, 0, 1, 0, 8),     # tensor-core FP16 mode: n outside 256 / 4096 / 65536
    (4096, 1, 1, 2, 0, 8),     # tensor-core BF16 mode: fp64 data
    (4096, 1, 0, 1, 0x2, 8),   # tensor-core mode with bit-reversed input
])
def test_plan_validation_without_gpu(L, n0, batch, dtype, mode, flags, status):
    import genfft_gb300 as G
    d = G.Desc(0, dtype, mode, flags, n0, 0, batch, 0, 0, 0, 0)
    h = ctypes.c_void_p()
    assert L.gfft_plan_create(ctypes.byref(h), ctypes.byref(d)) == status
    assert not h.value
    assert L.gfft_last_error()


def test_null_arguments(L):
    assert L.gfft_plan_create(None, None) == 2
    assert L.gfft_plan_destroy(None) == 10
    assert L.gfft_exec(None, 0, None, None, None) == 10
