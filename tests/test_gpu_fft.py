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


@pytest.mark.parametrize("tc", [0, 1], ids=["fma", "tensor-cores"])
@pytest.mark.parametrize("direction", [-1, 1])
def test_y246_lines_against_numpy(capi, tc, direction):
    """The elastic y transform of six spectra on the 246 = 6 x 41 engine,
    with the 41-point stage as FP32 multiply-adds or on the tensor cores
    (split-precision TF32), against numpy: within 3e-6 x log2(246) of the
    largest output."""
    import torch
    nx, nzc = 5, 10
    rng = np.random.default_rng(41 + tc)
    x = rng.standard_normal((6, nx, 246, nzc)) + 1j * rng.standard_normal((6, nx, 246, nzc))
    ref = np.fft.fft(x, axis=2) if direction < 0 else np.fft.ifft(x, axis=2) * 246
    d = torch.tensor(np.stack([x.real, x.imag], axis=-1), dtype=torch.float32, device="cuda").contiguous()
    s = torch.cuda.current_stream().cuda_stream
    lib = capi.load()
    assert lib.pfgb_fft_y246x6(tc, direction, nx, nzc, d.data_ptr(), s) == 0, lib.pfgb_last_error(None)
    torch.cuda.synchronize()
    got = d.cpu().numpy().astype(np.float64)
    got = got[..., 0] + 1j * got[..., 1]
    err = np.abs(got - ref).max()
    assert err <= 3e-6 * np.log2(246) * np.abs(ref).max(), err
