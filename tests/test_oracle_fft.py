"""The oracle's own FFT (stand-in for cuFFT) against numpy's pocketfft."""
import numpy as np
import pytest

SHAPES = [(8, 12, 10), (6, 5, 7), (16, 16, 16), (24, 20, 18), (41, 6, 82), (3, 2, 2), (12, 6, 246)]


@pytest.mark.parametrize("shape", SHAPES)
def test_r2c_matches_numpy(oracle, shape):
    import oracle_py
    rng = np.random.default_rng(1)
    x = rng.standard_normal(shape)
    k = oracle_py.fft_r2c(x)
    ref = np.fft.rfftn(x)
    assert np.abs(k - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("shape", SHAPES)
def test_c2r_roundtrip(oracle, shape):
    import oracle_py
    rng = np.random.default_rng(2)
    x = rng.standard_normal(shape)
    back = oracle_py.fft_c2r(oracle_py.fft_r2c(x), shape[2]) / x.size
    assert np.abs(back - x).max() <= 1e-13


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 41, 82, 123, 246, 64, 160])
def test_1d_against_numpy(oracle, n):
    import oracle_py
    import ctypes
    rng = np.random.default_rng(n)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex128)
    out = np.empty_like(x)
    oracle_py.lib().pfo_fft1d(n, -1, x.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p))
    assert np.abs(out - np.fft.fft(x)).max() <= 1e-13 * max(1.0, np.abs(x).sum())
    oracle_py.lib().pfo_fft1d(n, +1, x.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p))
    assert np.abs(out - np.fft.ifft(x) * n).max() <= 1e-13 * max(1.0, np.abs(x).sum())
