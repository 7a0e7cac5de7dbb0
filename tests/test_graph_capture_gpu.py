"""Plans captured into a CUDA graph and replayed give the same bits as
eager execution: the fused C2C, the persistent four-step, the three-pass
C2C and the 2D transform, whose kernels are programmatic dependent
launches (they start while the previous kernel drains and wait for it
before reading), captured as programmatic graph edges."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,n0,n1,batch", [("c2c", 1 << 12, 0, 64), ("c2c", 1 << 16, 0, 8),
                                              ("c2c", 1 << 22, 0, 2), ("c2d", 1024, 512, 2)])
def test_capture_replay_matches_eager(gfft, kind, n0, n1, batch):
    import torch
    g = torch.Generator(device="cuda").manual_seed(n0 + n1)
    shape = (batch, n1, n0) if kind == "c2d" else (batch, n0)
    x = torch.randn(*shape, dtype=torch.complex64, device="cuda", generator=g)
    if kind == "c2d":
        p = gfft.Plan(gfft.KIND_C2C_2D, gfft.F32, n0, n1, batch)
    else:
        p = gfft.Plan(gfft.KIND_C2C, gfft.F32, n0, 0, batch)
    y, z = torch.empty_like(x), torch.empty_like(x)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        p.exec(y, x, stream=s)            # warm-up: tables and workspaces exist before capture
        p.exec(z, y, True, stream=s)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    ye, ze = y.clone(), z.clone()
    y.zero_()
    z.zero_()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        p.exec(y, x)
        p.exec(z, y, True)
    for _ in range(2):
        graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(y, ye)
    assert torch.equal(z, ze)
    assert gfft.device_error() == 0
