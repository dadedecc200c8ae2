"""Oracle for the learned elastic warm start (test infrastructure only).

CPU restatement, in float64 numpy, of the Fourier neural operator that
predicts the heterogeneous displacement correction u - u_hom from
(phi, eta, eps0 x 6).  The model has no counterpart in the reference: the
reference warm-starts the heterogeneous elastic iteration from the previous
step's displacement (main_cuda.cu:28792-28870) and nothing else.  This file
restates the published FNO-3d (Li et al., "Fourier Neural Operator for
Parametric Partial Differential Equations", ICLR 2021) with the layout and
conventions the CUDA path uses, so that parity rests on:

- numpy.fft for the truncated spectral convolution, and
- central finite differences of this float64 forward for the gradients.

It is the oracle for the CUDA kernels, never the thing measured or shipped.

Model (width W = 32, hidden H = 64, IN = 8 inputs, OUT = 3 outputs):

    a_s  = in_scale * a                            (8 channels)
    v0   = P a_s + p                               (lift, W x 8)
    v_l+1 = act_l(K_l v_l + W_l v_l + b_l)         (l = 0..L-1; act = GELU,
                                                    identity on the last)
    K v  = irfftn( R(k) . rfftn(v, norm=forward) on the retained modes,
                   norm=forward )
    y    = out_scale * (Q2 GELU(Q1 v_L + q1) + q2) (projection, H x W, 3 x H)

Retained modes: kz in [0, m), and for x and y the two corner blocks
[0, m) and [N - m, N) (indices jx, jy in [0, 2m); j < m -> k = j, else
k = N - 2m + j).  Spectral weights R_l[i][o][mode] are complex, mode =
(jx * 2m + jy) * m + kz.  GELU is the exact erf form.

Weights P, W_l, R_l, Q1, Q2 are stored in bfloat16 on the GPU (master copy
float32); biases are float32.  ``round_weights`` rounds the weight blocks of
a flat parameter vector to bfloat16 (round to nearest, ties to even) so the
oracle evaluates the same weights the GPU does.

Loss: relative squared error  sum (y - t)^2 / sum t^2  over all outputs.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from math import sqrt

import numpy as np
from scipy.special import erf

WIDTH, HIDDEN, IN, OUT = 32, 64, 8, 3


@dataclass
class Config:
    Nx: int
    Ny: int
    Nz: int
    modes: int = 12
    layers: int = 4
    in_scale: np.ndarray = field(default_factory=lambda: np.ones(IN))
    out_scale: np.ndarray = field(default_factory=lambda: np.ones(OUT))

    @property
    def nmodes(self) -> int:
        return 4 * self.modes ** 3


def layout(cfg: Config):
    """(name, shape, is_weight) of each block of the flat parameter vector,
    in storage order."""
    W, H, M = WIDTH, HIDDEN, cfg.nmodes
    out = [("P", (W, IN), True), ("p", (W,), False)]
    for l in range(cfg.layers):
        out += [("W%d" % l, (W, W), True), ("b%d" % l, (W,), False), ("R%d" % l, (W, W, M, 2), True)]
    out += [("Q1", (H, W), True), ("q1", (H,), False), ("Q2", (OUT, H), True), ("q2", (OUT,), False)]
    return out


def num_params(cfg: Config) -> int:
    return sum(int(np.prod(s)) for _, s, _ in layout(cfg))


def unpack(flat: np.ndarray, cfg: Config) -> dict:
    d, o = {}, 0
    for name, shape, _ in layout(cfg):
        n = int(np.prod(shape))
        d[name] = np.asarray(flat[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    assert o == flat.size
    return d


def offsets(cfg: Config) -> dict:
    d, o = {}, 0
    for name, shape, _ in layout(cfg):
        d[name] = o
        o += int(np.prod(shape))
    return d


def bf16_round(x: np.ndarray) -> np.ndarray:
    """float32 -> bfloat16 -> float64, round to nearest, ties to even."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def round_weights(flat: np.ndarray, cfg: Config) -> np.ndarray:
    out = np.asarray(flat, dtype=np.float64).copy()
    o = 0
    for _, shape, is_w in layout(cfg):
        n = int(np.prod(shape))
        if is_w:
            out[o:o + n] = bf16_round(out[o:o + n])
        o += n
    return out


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / sqrt(2.0)))


def mode_index(n: int, m: int) -> np.ndarray:
    return np.concatenate([np.arange(m), np.arange(n - m, n)])


def spectral_conv(v: np.ndarray, R: np.ndarray, cfg: Config) -> np.ndarray:
    """v [W][X][Y][Z] -> irfftn(R . rfftn(v)) on the retained modes."""
    m = cfg.modes
    X, Y, Z = cfg.Nx, cfg.Ny, cfg.Nz
    V = np.fft.rfftn(v, axes=(1, 2, 3), norm="forward")
    ix, iy = mode_index(X, m), mode_index(Y, m)
    Vs = V[:, ix][:, :, iy][:, :, :, :m].reshape(WIDTH, -1)          # [i][mode]
    Rc = (R[..., 0] + 1j * R[..., 1])                                  # [i][o][mode]
    Os = np.einsum("im,iom->om", Vs, Rc).reshape(WIDTH, 2 * m, 2 * m, m)
    full = np.zeros((WIDTH, X, Y, Z // 2 + 1), dtype=np.complex128)
    full[np.ix_(np.arange(WIDTH), ix, iy, np.arange(m))] = Os
    return np.fft.irfftn(full, s=(X, Y, Z), axes=(1, 2, 3), norm="forward")


def forward(flat: np.ndarray, a: np.ndarray, cfg: Config) -> np.ndarray:
    """a [8][X][Y][Z] -> y [3][X][Y][Z] (float64)."""
    p = unpack(flat, cfg)
    a_s = a * np.asarray(cfg.in_scale, dtype=np.float64)[:, None, None, None]
    v = np.einsum("oi,ixyz->oxyz", p["P"], a_s) + p["p"][:, None, None, None]
    for l in range(cfg.layers):
        pre = spectral_conv(v, p["R%d" % l], cfg) + np.einsum("oi,ixyz->oxyz", p["W%d" % l], v) \
            + p["b%d" % l][:, None, None, None]
        v = gelu(pre) if l < cfg.layers - 1 else pre
    h = gelu(np.einsum("ji,ixyz->jxyz", p["Q1"], v) + p["q1"][:, None, None, None])
    y = np.einsum("cj,jxyz->cxyz", p["Q2"], h) + p["q2"][:, None, None, None]
    return y * np.asarray(cfg.out_scale, dtype=np.float64)[:, None, None, None]


def loss(flat: np.ndarray, a: np.ndarray, t: np.ndarray, cfg: Config) -> float:
    y = forward(flat, a, cfg)
    return float(np.sum((y - t) ** 2) / np.sum(t * t))


def fd_gradient(flat: np.ndarray, a: np.ndarray, t: np.ndarray, cfg: Config, idx, h: float = 1e-4):
    """Central differences of the loss for the parameters at ``idx``.  The
    perturbation is applied to the float64 value the forward reads (the
    gradient at the bfloat16 point, as the GPU computes it)."""
    g = np.empty(len(idx))
    for n, i in enumerate(idx):
        fp = flat.copy(); fp[i] += h
        fm = flat.copy(); fm[i] -= h
        g[n] = (loss(fp, a, t, cfg) - loss(fm, a, t, cfg)) / (2 * h)
    return g


def adam_reference(w, g, m, v, t, lr, b1, b2, eps, wd):
    """One Adam step with decoupled weight decay (Loshchilov & Hutter), the
    update the library applies to its float32 master weights."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    w = w - lr * (mh / (np.sqrt(vh) + eps) + wd * w)
    return w, m, v
