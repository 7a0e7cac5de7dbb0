"""Programmatic dependent launches (every kernel of a chain starts while the
previous one drains and waits for it before touching memory) against
ordinary launches (GFFT_PDL=0): the same kernels, so every path must give
the same bits.  A kernel that touched memory before its wait would race
with the previous kernel and show here.  Each mode runs in a subprocess
(the switch is read once per process)."""
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
g = torch.Generator(device="cuda").manual_seed(11)
outs = {}
# chains of dependent launches: forward then inverse, several sizes and paths
for n, b in [(1 << 10, 64), (1 << 12, 32), (1 << 14, 8), (1 << 15, 4), (1 << 20, 2), (1 << 22, 2)]:
    x = torch.randn(b, n, dtype=torch.complex64, device="cuda", generator=g)
    y = G.fft(x)
    outs[f"c2c_{n}"] = y.cpu().numpy()
    outs[f"c2c_inv_{n}"] = G.ifft(y).cpu().numpy()
x = torch.randn(2, 1024, 4096, dtype=torch.complex64, device="cuda", generator=g)
outs["c2d"] = G.fft2(x).cpu().numpy()
xr = torch.rand(1024, 4096, dtype=torch.float32, device="cuda", generator=g)
outs["r2d"] = G.rfft2(xr, half=True).cpu().numpy()
for n in (1 << 14, 1 << 20):
    xr1 = torch.rand(3, n, dtype=torch.float32, device="cuda", generator=g)
    f = G.rfft(xr1)
    outs[f"r2c_{n}"] = f.cpu().numpy()
    p = G.Plan(G.KIND_R2C, G.F32, n, 0, 3, G.FLAG_HALF_SPECTRUM)
    xb = torch.empty(3, n, dtype=torch.float32, device="cuda")
    p.exec(xb, f, True)
    outs[f"c2r_{n}"] = xb.cpu().numpy()
torch.cuda.synchronize()
assert G.device_error() == 0, "device-side timeout"
np.savez(sys.argv[1], **outs)
"""


def test_dependent_launches_match_ordinary_bitwise(gfft, tmp_path):
    res = {}
    for mode in ("pdl", "ordinary"):
        env = dict(os.environ)
        env["GFFT_PDL"] = "1" if mode == "pdl" else "0"
        out = str(tmp_path / f"{mode}.npz")
        r = subprocess.run([sys.executable, "-c", SCRIPT % ROOT, out], env=env, capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stderr[-3000:]
        res[mode] = np.load(out)
    for k in res["pdl"].files:
        a, b = res["pdl"][k], res["ordinary"][k]
        assert a.shape == b.shape, k
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), (k, np.max(np.abs(a - b)))
