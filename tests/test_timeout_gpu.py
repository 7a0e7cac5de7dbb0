"""Every device-side wait is bounded.  A persistent four-step launch whose
row tiles wait on column tiles that are never scheduled (a counter nothing
increments) must give up after its one-second bound, report the timeout
through the device error word (gfft_device_error: code 1,
GFFT_ERR_TIMEOUT), write nothing, and leave the context usable for the next
transform."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_stalled_wait_reports_timeout(gfft):
    import torch
    L = gfft.lib()
    L.gfft_test_stalled_fourstep.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.gfft_test_stalled_fourstep.restype = ctypes.c_int
    n = 1 << 16
    assert gfft.device_error() == 0
    x = torch.randn(1, n, dtype=torch.complex64, device="cuda")
    out = torch.full_like(x, 7.0)
    st = torch.cuda.current_stream()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(st)
    assert L.gfft_test_stalled_fourstep(out.data_ptr(), x.data_ptr(), st.cuda_stream) == 0
    t1.record(st)
    torch.cuda.synchronize()
    waited = t0.elapsed_time(t1)
    code = ctypes.c_int()
    assert L.gfft_device_error(ctypes.byref(code)) == 7  # GFFT_ERR_TIMEOUT
    assert code.value == 1
    assert 500.0 < waited < 10000.0, waited  # the bound, not a hang
    assert torch.all(out == 7.0)              # nothing written
    assert gfft.device_error() == 0           # reading reset it
    # the context still works
    y = gfft.fft(x)
    torch.cuda.synchronize()
    exact = np.fft.fft(x.cpu().numpy().astype(np.complex128))
    assert np.linalg.norm(y.cpu().numpy() - exact) / np.linalg.norm(exact) < 4e-6
