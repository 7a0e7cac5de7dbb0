"""Host-side rules of the torch.fft-compatible front end (no GPU needed):
the norm factors and the argument checks."""
import math

import pytest


def test_norm_factors():
    from genfft_gb300.torchfft import norm_scale
    n = 1024
    assert norm_scale(None, n, False) == 1.0 and norm_scale(None, n, True) == 1.0 / n
    assert norm_scale("backward", n, False) == 1.0 and norm_scale("backward", n, True) == 1.0 / n
    assert norm_scale("forward", n, False) == 1.0 / n and norm_scale("forward", n, True) == 1.0
    assert norm_scale("ortho", n, False) == norm_scale("ortho", n, True) == 1.0 / math.sqrt(n)
    with pytest.raises(ValueError):
        norm_scale("unitary", n, False)


def test_power_of_two_rule():
    from genfft_gb300.torchfft import _check_pow2
    for n in (1, 2, 1024, 1 << 22):
        _check_pow2(n, "n")
    for n in (0, 3, 100, 1000):
        with pytest.raises(ValueError):
            _check_pow2(n, "n")


def test_cpu_tensor_rejected():
    import torch
    from genfft_gb300 import torchfft
    with pytest.raises(ValueError):
        torchfft.fft(torch.zeros(4, 8, dtype=torch.complex64))
