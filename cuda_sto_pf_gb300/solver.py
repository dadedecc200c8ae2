"""Python host mirror of the reference's time-stepping driver, over the C ABI.

``Solver`` owns one pfgb context (one GPU).  Host arrays are numpy float64 in
the reference's C order [Nx][Ny][Nz].  Device arrays (torch tensors or raw
pointers) can be passed to ``load_device`` for runs that keep data resident.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data_as(ctypes.c_void_p)
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return ctypes.c_void_p(int(a))


class Solver:
    def __init__(self, params: capi.Params, device: int = 0):
        self.lib = capi.load()
        self.params = params
        self.ctx = ctypes.c_void_p()
        st = self.lib.pfgb_create(ctypes.byref(params), device, ctypes.byref(self.ctx))
        capi.check(st, "pfgb_create")
        self.shape = (params.Nx, params.Ny, params.Nz)
        self.N = params.Nx * params.Ny * params.Nz
        self.Nk = params.Nx * params.Ny * (params.Nz // 2 + 1)

    def close(self) -> None:
        if self.ctx:
            self.lib.pfgb_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, st, where):
        capi.check(st, where, self.ctx)

    def set_stream(self, stream_ptr: int) -> None:
        self._chk(self.lib.pfgb_set_stream(self.ctx, ctypes.c_void_p(stream_ptr)), "pfgb_set_stream")

    def load(self, phi, xB, eta=None, dYdt=None) -> None:
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
                for a in (phi, xB, eta, dYdt)]
        self._keep = arrs
        self._chk(self.lib.pfgb_load_fields(self.ctx, *[_ptr(a) for a in arrs]), "pfgb_load_fields")

    def load_device(self, phi, xB, eta=None, dYdt=None) -> None:
        self._chk(self.lib.pfgb_load_fields_device(self.ctx, _ptr(phi), _ptr(xB), _ptr(eta), _ptr(dYdt)),
                  "pfgb_load_fields_device")

    def step(self, nsteps: int = 1) -> capi.StepStats:
        st = capi.StepStats()
        self._chk(self.lib.pfgb_step(self.ctx, nsteps, ctypes.byref(st)), "pfgb_step")
        return st

    def minimize(self, n: int = 1, stats: capi.MinStats | None = None,
                 stop_on_convergence: bool = False) -> capi.MinStats:
        st = stats if stats is not None else capi.MinStats()
        self._chk(self.lib.pfgb_minimize(self.ctx, n, 1 if stop_on_convergence else 0, ctypes.byref(st)),
                  "pfgb_minimize")
        return st

    def checkpoint_save(self, path: str, initial_state_class=None, fixture_manifest_sha256=None,
                        profile_library_manifest_sha256=None) -> None:
        """pfgb_checkpoint_save: the reference's zero-mode checkpoint file."""
        enc = lambda v: None if v is None else v.encode()
        self._chk(self.lib.pfgb_checkpoint_save(self.ctx, path.encode(), enc(initial_state_class),
                                                enc(fixture_manifest_sha256), enc(profile_library_manifest_sha256)),
                  "pfgb_checkpoint_save")

    def checkpoint_restore(self, path: str, initial_state_class=None, fixture_manifest_sha256=None,
                           profile_library_manifest_sha256=None) -> None:
        """pfgb_checkpoint_restore: continue from a zero-mode checkpoint."""
        enc = lambda v: None if v is None else v.encode()
        self._chk(self.lib.pfgb_checkpoint_restore(self.ctx, path.encode(), enc(initial_state_class),
                                                   enc(fixture_manifest_sha256),
                                                   enc(profile_library_manifest_sha256)),
                  "pfgb_checkpoint_restore")

    def set_warm_start_model(self, model) -> None:
        """Attach a ``fno.WarmStartModel`` (None detaches); it is used when
        elastic_warm_start_source is 1 or 2."""
        self._model = model
        self._chk(self.lib.pfgb_set_warm_start_model(self.ctx, model.handle if model is not None else None),
                  "pfgb_set_warm_start_model")

    def training_pair(self, d_in8, d_target3) -> capi.StepStats:
        """Cold elastic solve on the current fields; writes the model inputs
        [8][N] and the correction u - u_hom [3][N] into device float32 buffers."""
        st = capi.StepStats()
        self._chk(self.lib.pfgb_elastic_training_pair(self.ctx, _ptr(d_in8), _ptr(d_target3), ctypes.byref(st)),
                  "pfgb_elastic_training_pair")
        return st

    def step_nostats(self, nsteps: int = 1) -> None:
        self._chk(self.lib.pfgb_step(self.ctx, nsteps, None), "pfgb_step")

    def fields(self) -> dict:
        out = {k: np.empty(self.shape) for k in ("phi", "xB", "Y", "eta", "dYdt")}
        self._chk(self.lib.pfgb_read_fields(self.ctx, *[_ptr(out[k]) for k in ("phi", "xB", "Y", "eta", "dYdt")]),
                  "pfgb_read_fields")
        return out

    def elastic(self) -> dict:
        sig = np.empty((6,) + self.shape, dtype=np.float32)
        eps = np.empty((6,) + self.shape, dtype=np.float32)
        self._chk(self.lib.pfgb_read_elastic(self.ctx, _ptr(sig), _ptr(eps)), "pfgb_read_elastic")
        return {"sigma": sig, "strain": eps}

    def displacement_k(self) -> np.ndarray:
        u = np.empty((3, self.Nk, 2), dtype=np.float32)
        self._chk(self.lib.pfgb_read_displacement_k(self.ctx, _ptr(u)), "pfgb_read_displacement_k")
        return u[..., 0] + 1j * u[..., 1]

    def diagnostics(self) -> capi.Diag:
        d = capi.Diag()
        self._chk(self.lib.pfgb_diagnostics(self.ctx, ctypes.byref(d)), "pfgb_diagnostics")
        return d

    def sync(self) -> None:
        self._chk(self.lib.pfgb_sync(self.ctx), "pfgb_sync")

    def device_bytes(self) -> int:
        return int(self.lib.pfgb_device_bytes(self.ctx))

    # --- instrumentation ---------------------------------------------------
    def profile_enable(self, on: bool = True) -> None:
        self._chk(self.lib.pfgb_profile_enable(self.ctx, 1 if on else 0), "pfgb_profile_enable")

    def launches(self) -> int:
        return int(self.lib.pfgb_profile_launches(self.ctx))

    def profile_read(self) -> list:
        n = self.lib.pfgb_profile_read(self.ctx, None, None, None, None, 0)
        if n <= 0:
            return []
        names = (ctypes.c_char_p * n)()
        ms = (ctypes.c_double * n)()
        by = (ctypes.c_double * n)()
        cnt = (ctypes.c_int * n)()
        self.lib.pfgb_profile_read(self.ctx, names, ms, by, cnt, n)
        return [{"kernel": names[i].decode(), "ms": ms[i], "bytes": by[i], "launches": cnt[i]} for i in range(n)]

    def set_fields(self, phi, xB, eta=None, dYdt=None) -> None:
        """Replace the fields from host buffers, keeping solver history."""
        self._chk(self.lib.pfgb_set_fields(self.ctx, _ptr(phi), _ptr(xB), _ptr(eta), _ptr(dYdt)),
                  "pfgb_set_fields")

    def read_into(self, phi=None, xB=None, Y=None, eta=None, dYdt=None) -> None:
        """Read fields into caller-owned (e.g. pinned) float64 host buffers."""
        self._chk(self.lib.pfgb_read_fields(self.ctx, _ptr(phi), _ptr(xB), _ptr(Y), _ptr(eta), _ptr(dYdt)),
                  "pfgb_read_fields")

