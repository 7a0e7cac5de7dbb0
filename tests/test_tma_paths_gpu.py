"""The persistent TMA-pipelined tile kernels against the plain tile kernels:
the same Stockham arithmetic on the same twiddles, so outputs must be
bit-identical.  The plain path is forced in a subprocess with GFFT_NO_TMA=1.
No device-side wait may time out."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys, numpy as np, torch
sys.path.insert(0, %r)
import genfft_gb300 as G
g = torch.Generator(device="cuda").manual_seed(5)
outs = {}
for (dt, n, b) in [(torch.complex64, 1 << 15, 3), (torch.complex64, 1 << 22, 2), (torch.complex64, 1 << 16, 5),
                   (torch.complex128, 1 << 16, 3), (torch.complex128, 1 << 18, 2)]:
    x = torch.randn(b, n, dtype=dt, device="cuda", generator=g)
    outs[f"c2c_{n}_{dt}"] = G.fft(x).cpu().numpy()
    outs[f"c2ci_{n}_{dt}"] = G.ifft(x).cpu().numpy()
x = torch.randn(2, 1024, 512, dtype=torch.complex64, device="cuda", generator=g)
outs["c2d"] = G.fft2(x).cpu().numpy()
xr = torch.rand(1024, 2048, dtype=torch.float32, device="cuda", generator=g)
outs["r2d_full"] = G.rfft2(xr).cpu().numpy()
outs["r2d_half"] = G.rfft2(xr, half=True).cpu().numpy()
xr1 = torch.rand(3, 1 << 20, dtype=torch.float32, device="cuda", generator=g)
outs["r2c"] = G.rfft(xr1).cpu().numpy()
torch.cuda.synchronize()
assert G.device_error() == 0, "device-side timeout"
np.savez(sys.argv[1], **outs)
"""


def test_tma_matches_plain_bitwise(gfft, tmp_path):
    res = {}
    for mode in ("tma", "plain"):
        env = dict(os.environ)
        env["GFFT_3PASS"] = "0"  # 2^22 through the two-pass tiles in both modes
        if mode == "plain":
            env["GFFT_NO_TMA"] = "1"
        out = str(tmp_path / f"{mode}.npz")
        r = subprocess.run([sys.executable, "-c", SCRIPT % ROOT, out], env=env, capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stderr[-3000:]
        res[mode] = np.load(out)
    for k in res["tma"].files:
        a, b = res["tma"][k], res["plain"][k]
        assert a.shape == b.shape, k
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), (k, np.max(np.abs(a - b)))
