"""The oracle's restatement of the reference's FFT ocean (no GPU): the
butterfly passes compute the inverse DFT of the h(k,t) field (up to the
binary16 weights the reference uses), heights are real fields, and the
sea-state parameters follow OpenGLRealOcean."""
import numpy as np
import pytest

from stonefish_gb300 import abi


def params(passes=6, state=1.0):
    p = abi.FftOceanParams()
    p.wind = state * 5.0 + 2.0
    p.omega = 5.0 * np.exp(-state) + 0.2
    p.amplitude = 1.0
    p.km = 370.0
    p.cm = 0.23
    for i, g in enumerate((893.0, 101.0, 21.0, 11.0)):
        p.grid_sizes[i] = g
    p.passes = passes
    p.propagate = 1
    return p


@pytest.mark.parametrize("t", [0.0, 3.7])
def test_butterfly_passes_are_the_inverse_dft(oracle, t):
    p = params(passes=6)
    h0 = oracle.fft_ocean(p, t, init_only=True).astype(np.float64)
    out = oracle.fft_ocean(p, t).astype(np.float64)
    N = 1 << p.passes
    for pair in range(2):
        z = h0[:, :, 2 * pair] + 1j * h0[:, :, 2 * pair + 1]
        ref = np.fft.ifft2(z) * N * N               # unnormalised inverse transform
        got = out[:, :, 2 * pair] + 1j * out[:, :, 2 * pair + 1]
        scale = np.max(np.abs(ref))
        # binary16 twiddle factors: measured 2e-4 to 5e-4 of the field's maximum
        assert np.max(np.abs(got - ref)) < 2e-3 * scale, (pair, np.max(np.abs(got - ref)) / scale)


def test_fields_are_seeded_and_time_dependent(oracle):
    p = params(passes=6)
    a = oracle.fft_ocean(p, 1.0)
    b = oracle.fft_ocean(p, 1.0)
    c = oracle.fft_ocean(p, 2.0)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)
    assert np.all(np.isfinite(a)) and np.max(np.abs(a[:, :, 0])) > 0.0


def test_higher_sea_state_gives_higher_waves(oracle):
    lo = oracle.fft_ocean(params(passes=6, state=0.5), 0.0)
    hi = oracle.fft_ocean(params(passes=6, state=3.0), 0.0)
    assert np.std(hi[:, :, 0]) > np.std(lo[:, :, 0])
