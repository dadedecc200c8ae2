"""Learned start of the heterogeneous elastic iteration, over the C ABI.

``WarmStartModel`` owns one pfgb_fno (a Fourier neural operator with
bfloat16 weights on one GPU).  Device tensors are float32, channel-major
[C][Nx][Ny][Nz], passed as torch CUDA tensors or raw pointers; the model
never copies them.  ``make_pairs`` builds training pairs with the solver's
own cold elastic solve, ``train`` fits the model with Adam, and
``Solver.set_warm_start_model`` plugs it in at the solver's warm-start
point.  The reference has no such model: its heterogeneous iteration starts
from the previous step's displacement (main_cuda.cu:28792-28870).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import capi


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)
    return ctypes.c_void_p(int(a))


class WarmStartModel:
    def __init__(self, shape, modes: int = 12, layers: int = 4, seed: int = 20240611, device: int = 0,
                 in_scale=None, out_scale=None, _handle=None):
        self.lib = capi.load()
        self.handle = ctypes.c_void_p()
        if _handle is not None:
            self.handle = _handle
        else:
            cfg = capi.FnoConfig()
            self.lib.pfgb_fno_config_default(ctypes.byref(cfg))
            cfg.Nx, cfg.Ny, cfg.Nz = shape
            cfg.modes, cfg.layers, cfg.seed = modes, layers, seed
            if in_scale is not None:
                for i, v in enumerate(in_scale):
                    cfg.in_scale[i] = float(v)
            if out_scale is not None:
                for i, v in enumerate(out_scale):
                    cfg.out_scale[i] = float(v)
            capi.check(self.lib.pfgb_fno_create(ctypes.byref(cfg), device, ctypes.byref(self.handle)),
                       "pfgb_fno_create")
        c = self.config()
        self.shape = (c.Nx, c.Ny, c.Nz)
        self.N = c.Nx * c.Ny * c.Nz

    @classmethod
    def load(cls, path: str, shape=None, device: int = 0) -> "WarmStartModel":
        lib = capi.load()
        h = ctypes.c_void_p()
        nx, ny, nz = shape if shape is not None else (0, 0, 0)
        capi.check(lib.pfgb_fno_load(path.encode(), nx, ny, nz, device, ctypes.byref(h)), "pfgb_fno_load")
        return cls(None, _handle=h)

    def close(self) -> None:
        if self.handle:
            self.lib.pfgb_fno_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def config(self) -> capi.FnoConfig:
        c = capi.FnoConfig()
        capi.check(self.lib.pfgb_fno_get_config(self.handle, ctypes.byref(c)), "pfgb_fno_get_config")
        return c

    def set_scales(self, in_scale=None, out_scale=None) -> None:
        i = None if in_scale is None else (ctypes.c_float * 8)(*[float(v) for v in in_scale])
        o = None if out_scale is None else (ctypes.c_float * 3)(*[float(v) for v in out_scale])
        capi.check(self.lib.pfgb_fno_set_scales(self.handle, i, o), "pfgb_fno_set_scales")

    def set_stream(self, stream_ptr: int) -> None:
        capi.check(self.lib.pfgb_fno_set_stream(self.handle, ctypes.c_void_p(stream_ptr)), "pfgb_fno_set_stream")

    @property
    def num_params(self) -> int:
        return int(self.lib.pfgb_fno_num_params(self.handle))

    def params(self) -> np.ndarray:
        h = np.empty(self.num_params, dtype=np.float32)
        capi.check(self.lib.pfgb_fno_get_params(self.handle, _ptr(h), h.size), "pfgb_fno_get_params")
        return h

    def set_params(self, h) -> None:
        h = np.ascontiguousarray(h, dtype=np.float32)
        capi.check(self.lib.pfgb_fno_set_params(self.handle, _ptr(h), h.size), "pfgb_fno_set_params")

    def grad(self) -> np.ndarray:
        h = np.empty(self.num_params, dtype=np.float32)
        capi.check(self.lib.pfgb_fno_get_grad(self.handle, _ptr(h), h.size), "pfgb_fno_get_grad")
        return h

    def forward(self, d_in, d_out) -> None:
        capi.check(self.lib.pfgb_fno_forward(self.handle, _ptr(d_in), _ptr(d_out)), "pfgb_fno_forward")

    def loss_grad(self, d_in, d_target, accumulate: bool = False, want_loss: bool = True):
        loss = ctypes.c_double(float("nan"))
        capi.check(self.lib.pfgb_fno_loss_grad(self.handle, _ptr(d_in), _ptr(d_target), 1 if accumulate else 0,
                                               ctypes.byref(loss) if want_loss else None), "pfgb_fno_loss_grad")
        return loss.value if want_loss else None

    def adam_step(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
                  weight_decay: float = 0.0, clip_norm: float = 0.0) -> None:
        o = capi.FnoAdam(lr, beta1, beta2, eps, weight_decay, clip_norm)
        capi.check(self.lib.pfgb_fno_adam_step(self.handle, ctypes.byref(o)), "pfgb_fno_adam_step")

    def save(self, path: str) -> None:
        capi.check(self.lib.pfgb_fno_save(self.handle, path.encode()), "pfgb_fno_save")


def channel_scales(inputs, targets):
    """1 / RMS of each input channel, and the RMS of each target channel
    (over a device tensor batch [P][C][N]); the model is fitted in these
    units."""
    import torch
    with torch.no_grad():
        si = torch.zeros(inputs.shape[1], dtype=torch.float64, device=inputs.device)
        st = torch.zeros(targets.shape[1], dtype=torch.float64, device=targets.device)
        for i in range(inputs.shape[0]):   # one pair at a time: no full-size float64 copy
            si += inputs[i].double().pow(2).sum(dim=1)
            st += targets[i].double().pow(2).sum(dim=1)
        cnt = float(inputs.shape[0] * inputs.shape[2])
        i_rms = (si / cnt).sqrt().cpu().numpy()
        t_rms = (st / cnt).sqrt().cpu().numpy()
    in_scale = np.where(i_rms > 0, 1.0 / np.maximum(i_rms, 1e-30), 1.0)
    out_scale = np.where(t_rms > 0, t_rms, 1.0)
    return in_scale, out_scale


def make_pairs(solver, microstructures, inputs, targets) -> list:
    """For each (phi, xB, eta) in ``microstructures`` load it into ``solver``
    and write the training pair into inputs[i] / targets[i] (device float32
    tensors [P][8][N] / [P][3][N]).  Returns the cold-solve iteration counts."""
    its = []
    for i, (phi, xB, eta) in enumerate(microstructures):
        solver.load(phi, xB, eta)
        st = solver.training_pair(inputs[i], targets[i])
        its.append(int(st.elastic_iterations))
    return its


def train(model: WarmStartModel, inputs, targets, steps: int, lr: float = 1e-3, lr_final: float = 1e-5,
          clip_norm: float = 1.0, seed: int = 0, log_every: int = 0, log=print) -> list:
    """Adam over single pairs in a seeded random order, cosine learning-rate
    decay from lr to lr_final.  Returns the loss of each step."""
    rng = np.random.default_rng(seed)
    P = inputs.shape[0]
    order = np.concatenate([rng.permutation(P) for _ in range(steps // P + 1)])[:steps]
    losses = []
    for s, i in enumerate(order):
        loss = model.loss_grad(inputs[int(i)], targets[int(i)])
        a = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * s / max(1, steps - 1)))
        model.adam_step(a, clip_norm=clip_norm)
        losses.append(loss)
        if log_every and (s + 1) % log_every == 0:
            log("step %d loss %.4e (last %d mean %.4e)" % (s + 1, loss, log_every, np.mean(losses[-log_every:])))
    return losses
