"""Own 3D FFT kernels (no cuFFT) against numpy, through the C ABI."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(8, 12, 10), (16, 16, 16), (24, 20, 18), (41, 6, 82), (12, 6, 246), (64, 64, 64),
          (30, 28, 26), (5, 7, 4), (1, 3, 6)]


def _run(capi, prec, shape, x):
    import torch
    lib = capi.load()
    nx, ny, nz = shape
    dt = torch.float64 if prec == 0 else torch.float32
    d_in = torch.tensor(x, device="cuda", dtype=dt)
    d_k = torch.empty((nx, ny, nz // 2 + 1, 2), device="cuda", dtype=dt)
    s = torch.cuda.current_stream().cuda_stream
    assert lib.pfgb_fft3d_r2c(prec, nx, ny, nz, d_in.data_ptr(), d_k.data_ptr(), s) == 0
    k = d_k.cpu().numpy().astype(np.float64)
    k = k[..., 0] + 1j * k[..., 1]
    d_back = torch.empty((nx, ny, nz), device="cuda", dtype=dt)
    assert lib.pfgb_fft3d_c2r(prec, nx, ny, nz, d_k.data_ptr(), d_back.data_ptr(), s) == 0
    torch.cuda.synchronize()
    return k, d_back.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 3e-6)])
@pytest.mark.parametrize("shape", SHAPES)
def test_r2c_c2r_against_numpy(capi, shape, prec, tol):
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(shape)
    k, back = _run(capi, prec, shape, x)
    ref = np.fft.rfftn(x)
    assert np.abs(k - ref).max() <= tol * np.abs(ref).max() * np.log2(x.size + 1)
    assert np.abs(back / x.size - x).max() <= tol * np.abs(x).max() * np.log2(x.size + 1)


def test_fft_rejects_bad_size(capi):
    lib = capi.load()
    assert lib.pfgb_fft3d_r2c(0, 0, 4, 4, 1, 1, None) == 1
    assert lib.pfgb_fft3d_r2c(0, 4, 4, 4, None, 1, None) == 1
