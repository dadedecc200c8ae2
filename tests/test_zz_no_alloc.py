"""pfgb_fft3d_r2c_noalloc: the forward transform with its twiddle tables in
a static device array.  Compared with pfgb_fft3d_r2c on the same inputs; the
file is collected last so it also runs after every other GPU test."""
import ctypes

import numpy as np
import pytest

TOL = {0: 1e-13, 1: 3e-6}   # relative to max |X|, times log2(N+1)


# Stand-ins for device pointers in the refusal tests: every refusal below
# happens on the host before any CUDA call, so nothing dereferences them.
A, B = 0x1000, 0x2000


def test_noalloc_rejects_oversized_scratch(capi):
    lib = capi.load()
    # FP64 needs 16*(Nx+Ny+Nz) bytes (each axis padded to 256 B) > 32768
    assert lib.pfgb_fft3d_r2c_noalloc(0, 1024, 1024, 64, A, B, None) == 1
    assert b"twiddle scratch" in lib.pfgb_last_error(None)
    # bad precision / null buffers / bad size are refused before any launch
    assert lib.pfgb_fft3d_r2c_noalloc(2, 8, 8, 8, A, B, None) == 1
    assert lib.pfgb_fft3d_r2c_noalloc(0, 8, 8, 8, None, B, None) == 1
    assert lib.pfgb_fft3d_r2c_noalloc(1, 8, 8, 1, A, B, None) == 1


def test_transforms_reject_misaligned_buffers(capi):
    # the line engines copy 16-byte units from the buffers' base addresses:
    # a buffer off a 16-byte boundary is refused on the host, never launched
    lib = capi.load()
    for fn in (lib.pfgb_fft3d_r2c, lib.pfgb_fft3d_c2r, lib.pfgb_fft3d_r2c_noalloc):
        for prec in (0, 1):
            assert fn(prec, 12, 6, 246, A + 8, B, None) == 1
            assert b"16-byte aligned" in lib.pfgb_last_error(None)
            assert fn(prec, 12, 6, 246, A, B + 4, None) == 1


def _pair(lib, torch, prec, shape, seed):
    nx, ny, nz = shape
    dt = torch.float64 if prec == 0 else torch.float32
    x = np.random.default_rng(seed).standard_normal(shape)
    d_in = torch.tensor(x, device="cuda", dtype=dt)
    ref = torch.empty((nx, ny, nz // 2 + 1, 2), device="cuda", dtype=dt)
    got = torch.full_like(ref, float("nan"))
    s = torch.cuda.current_stream().cuda_stream
    assert lib.pfgb_fft3d_r2c(prec, nx, ny, nz, d_in.data_ptr(), ref.data_ptr(), s) == 0
    assert lib.pfgb_fft3d_r2c_noalloc(prec, nx, ny, nz, d_in.data_ptr(), got.data_ptr(), s) == 0, \
        lib.pfgb_last_error(None)
    torch.cuda.synchronize()
    return ref.cpu().numpy().astype(np.float64), got.cpu().numpy().astype(np.float64), x.size


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_matches_allocating_transform(capi, prec):
    import torch
    lib = capi.load()
    # two calls in a row with different sizes (the second rewrites the
    # tables of the first), then the first size again
    shapes = [(41, 6, 82), (24, 20, 18), (41, 6, 82), (64, 64, 64)]
    if prec == 1:
        # 246-long axes run the 6x41 engine in FP32: z of 246, and x / y of
        # 246 with an even Nz/2+1 (the strided-axis engine)
        shapes += [(12, 6, 246), (246, 6, 10), (6, 246, 10)]
    for i, shape in enumerate(shapes):
        ref, got, n = _pair(lib, torch, prec, shape, 100 + i)
        assert np.isfinite(got).all()
        err = np.abs(got - ref).max()
        assert err <= TOL[prec] * np.abs(ref).max() * np.log2(n + 1), (shape, err)


@pytest.mark.gpu
def test_noalloc_largest_fp32_table(capi):
    import torch
    lib = capi.load()
    # FP32 tables for 1024 + 1024 + 2 points fill 16640 of the 32768 bytes
    ref, got, n = _pair(lib, torch, 1, (1024, 1024, 2), 7)
    assert np.abs(got - ref).max() <= TOL[1] * np.abs(ref).max() * np.log2(n + 1)
