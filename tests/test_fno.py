"""Learned start of the heterogeneous elastic iteration.

The CUDA FNO against its float64 oracle (forward; gradients against central
finite differences of the oracle; the Adam update), model files, and the
solver hook at the warm-start point (main_cuda.cu:28792-28870): the plain
fixed point still runs to the residual tolerance, so the converged fields
do not depend on the start.  The model has no reference counterpart; its
oracle restates the published FNO-3d."""
import os
import sys

import numpy as np
import pytest

from conftest import REPO, params_for, rel_l2

sys.path.insert(0, os.path.join(REPO, "oracle"))
import fno_oracle as fo  # noqa: E402


def _cfg(shape, modes, layers, rng):
    return fo.Config(*shape, modes=modes, layers=layers, in_scale=rng.uniform(0.5, 2.0, 8),
                     out_scale=rng.uniform(0.5, 2.0, 3))


def _weights(cfg, rng, spread=0.3):
    w = rng.uniform(-spread, spread, fo.num_params(cfg)).astype(np.float32)
    # smaller spectral weights, as the library initialises them
    off = 0
    for name, shape, _ in fo.layout(cfg):
        n = int(np.prod(shape))
        if name.startswith("R"):
            w[off:off + n] *= 0.1
        off += n
    return w


# ---------------------------------------------------------------------------
# CPU: the oracle itself
# ---------------------------------------------------------------------------
def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.normal(size=4000), rng.uniform(-1e-3, 1e-3, 1000)]).astype(np.float32)
    # exact ties: low 16 bits 0x8000 with even and odd kept parts
    ties = (np.arange(64, dtype=np.uint32) << 16 | 0x8000 | 0x3F800000).view(np.float32)
    x = np.concatenate([x, ties, -ties])
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(fo.bf16_round(x), ref)


def test_oracle_spectral_conv_is_the_truncated_dft():
    """irfftn(R . rfftn(v)) on the corner blocks equals the direct sums over
    the retained wavenumbers (the form the kernels evaluate)."""
    rng = np.random.default_rng(2)
    X, Y, Z, m = 6, 8, 10, 2
    cfg = fo.Config(X, Y, Z, modes=m, layers=1)
    v = rng.normal(size=(fo.WIDTH, X, Y, Z))
    R = rng.normal(size=(fo.WIDTH, fo.WIDTH, 4 * m ** 3, 2))
    got = fo.spectral_conv(v, R, cfg)
    kx = fo.mode_index(X, m)
    ky = fo.mode_index(Y, m)
    x, y, z = np.arange(X), np.arange(Y), np.arange(Z)
    Ex = np.exp(-2j * np.pi * np.outer(kx, x) / X)
    Ey = np.exp(-2j * np.pi * np.outer(ky, y) / Y)
    Ez = np.exp(-2j * np.pi * np.outer(np.arange(m), z) / Z)
    C = np.einsum("cxyz,ax,by,kz->cabk", v, Ex, Ey, Ez) / (X * Y * Z)
    O = np.einsum("iabk,ioabk->oabk", C, (R[..., 0] + 1j * R[..., 1]).reshape(fo.WIDTH, fo.WIDTH, 2 * m, 2 * m, m))
    w = np.array([1.0] + [2.0] * (m - 1))
    want = np.real(np.einsum("oabk,ax,by,kz->oxyz", O * w, Ex.conj(), Ey.conj(), Ez.conj()))
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_oracle_is_translation_equivariant():
    """Periodic shifts of the inputs shift the prediction (size-independent
    property of the operator)."""
    rng = np.random.default_rng(3)
    cfg = _cfg((8, 8, 10), 3, 2, rng)
    w = fo.round_weights(_weights(cfg, rng), cfg)
    a = rng.normal(size=(8, 8, 8, 10))
    y = fo.forward(w, a, cfg)
    ys = fo.forward(w, np.roll(a, (2, 5, 3), axis=(1, 2, 3)), cfg)
    assert np.abs(np.roll(y, (2, 5, 3), axis=(1, 2, 3)) - ys).max() <= 1e-10 * np.abs(y).max()


# ---------------------------------------------------------------------------
# GPU: kernels against the oracle
# ---------------------------------------------------------------------------
def _dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).cuda()


def _model(capi, cfg, w):
    from cuda_sto_pf_gb300.fno import WarmStartModel
    m = WarmStartModel((cfg.Nx, cfg.Ny, cfg.Nz), modes=cfg.modes, layers=cfg.layers,
                       in_scale=cfg.in_scale, out_scale=cfg.out_scale)
    assert m.num_params == fo.num_params(cfg)
    m.set_params(w)
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("shape,modes,layers", [((8, 10, 12), 3, 4), ((6, 8, 300), 2, 2), ((16, 16, 16), 8, 1)])
def test_forward_matches_oracle(capi, shape, modes, layers):
    import torch
    rng = np.random.default_rng(10 + modes)
    cfg = _cfg(shape, modes, layers, rng)
    w = _weights(cfg, rng)
    a = rng.normal(size=(8,) + shape)
    with _model(capi, cfg, w) as m:
        out = torch.empty((3,) + shape, device="cuda")
        m.forward(_dev(a), out)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        # the bfloat16 copy is what the kernels read
        assert np.array_equal(m.params(), w)
    want = fo.forward(fo.round_weights(w, cfg), a, cfg)
    assert rel_l2(got, want) <= 2e-6


@pytest.mark.gpu
def test_gradients_match_finite_differences(capi):
    rng = np.random.default_rng(20)
    cfg = _cfg((8, 10, 12), 3, 3, rng)
    w = _weights(cfg, rng)
    wr = fo.round_weights(w, cfg)
    a = rng.normal(size=(8, 8, 10, 12))
    t = rng.normal(size=(3, 8, 10, 12))
    with _model(capi, cfg, w) as m:
        loss = m.loss_grad(_dev(a), _dev(t))
        g = m.grad()
    assert abs(loss - fo.loss(wr, a, t, cfg)) <= 1e-5 * fo.loss(wr, a, t, cfg)
    off = fo.offsets(cfg)
    for name, shape, _ in fo.layout(cfg):
        n = int(np.prod(shape))
        idx = off[name] + rng.choice(n, size=min(6, n), replace=False)
        fd = fo.fd_gradient(wr, a, t, cfg, idx, h=1e-4)
        scale = max(np.abs(fd).max(), 1e-6)
        assert np.abs(g[idx] - fd).max() <= 2e-3 * scale, (name, g[idx], fd)


@pytest.mark.gpu
def test_gradient_accumulates_over_pairs(capi):
    rng = np.random.default_rng(21)
    cfg = _cfg((8, 8, 8), 2, 2, rng)
    w = _weights(cfg, rng)
    a1, a2 = rng.normal(size=(2, 8, 8, 8, 8))
    t1, t2 = rng.normal(size=(2, 3, 8, 8, 8))
    with _model(capi, cfg, w) as m:
        m.loss_grad(_dev(a1), _dev(t1))
        g1 = m.grad()
        m.loss_grad(_dev(a2), _dev(t2))
        g2 = m.grad()
        m.loss_grad(_dev(a1), _dev(t1))
        m.loss_grad(_dev(a2), _dev(t2), accumulate=True)
        g12 = m.grad()
    assert np.abs(g12 - (g1 + g2)).max() <= 1e-5 * np.abs(g1 + g2).max()


@pytest.mark.gpu
def test_adam_step_matches_reference(capi):
    rng = np.random.default_rng(22)
    cfg = _cfg((8, 8, 8), 2, 1, rng)
    w = _weights(cfg, rng)
    a = rng.normal(size=(8, 8, 8, 8))
    t = rng.normal(size=(3, 8, 8, 8))
    lr, b1, b2, eps, wd = 1e-2, 0.9, 0.99, 1e-8, 1e-3
    mm = np.zeros(w.size)
    vv = np.zeros(w.size)
    ww = w.astype(np.float64)
    with _model(capi, cfg, w) as m:
        for step in (1, 2):
            m.loss_grad(_dev(a), _dev(t))
            g = m.grad().astype(np.float64)
            m.adam_step(lr, b1, b2, eps, wd)
            ww, mm, vv = fo.adam_reference(ww, g, mm, vv, step, lr, b1, b2, eps, wd)
            got = m.params()
            assert np.abs(got - ww).max() <= 2e-6 * max(1.0, np.abs(ww).max()), step


@pytest.mark.gpu
def test_save_load_roundtrip(capi, tmp_path):
    import torch
    from cuda_sto_pf_gb300.fno import WarmStartModel
    rng = np.random.default_rng(23)
    cfg = _cfg((8, 8, 12), 3, 2, rng)
    w = _weights(cfg, rng)
    a = _dev(rng.normal(size=(8, 8, 8, 12)))
    path = str(tmp_path / "model.pfgbfno")
    o1 = torch.empty((3, 8, 8, 12), device="cuda")
    o2 = torch.empty_like(o1)
    with _model(capi, cfg, w) as m:
        m.forward(a, o1)
        m.save(path)
    with WarmStartModel.load(path) as m2:
        c = m2.config()
        assert (c.Nx, c.Ny, c.Nz, c.modes, c.layers) == (8, 8, 12, 3, 2)
        assert np.allclose(list(c.in_scale), cfg.in_scale, rtol=1e-7)
        m2.forward(a, o2)
        assert np.array_equal(m2.params(), w)
    torch.cuda.synchronize()
    assert torch.equal(o1, o2)
    # the same weights on another grid
    with WarmStartModel.load(path, shape=(12, 10, 16)) as m3:
        assert m3.shape == (12, 10, 16)
    bad = tmp_path / "bad.pfgbfno"
    bad.write_bytes(b"not a model")
    with pytest.raises(capi.PfgbError):
        WarmStartModel.load(str(bad))


@pytest.mark.gpu
def test_invalid_model_configs_are_refused(capi):
    from cuda_sto_pf_gb300.fno import WarmStartModel
    with pytest.raises(capi.PfgbError):
        WarmStartModel((16, 16, 16), modes=9)       # 2 * modes > 16
    with pytest.raises(capi.PfgbError):
        WarmStartModel((16, 16, 16), modes=4, layers=0)


# ---------------------------------------------------------------------------
# GPU: the solver hook
# ---------------------------------------------------------------------------
def _micro(n, seed, count=4):
    """Seeded microstructure under the reference's raw-field rules (xB
    clamped to xB_max_safe = 0.07, main_cuda.cu:2904-2990)."""
    import ctypes
    from cuda_sto_pf_gb300 import capi, workloads
    w = workloads.ellipsoid_population(n=n, count=count, median_r=4.0, eta_sites=2, eta_r=2.5, seed=seed)
    phi, xB, eta = w["phi"], w["xB"], w["eta"]
    p = capi.default_params()
    capi.check(capi.load().pfgb_prepare_raw_fields(ctypes.byref(p), 0.07, phi.ctypes.data, xB.ctypes.data,
                                                   eta.ctypes.data, None, phi.size), "pfgb_prepare_raw_fields")
    return phi, xB, eta


def _params(capi, n, **kw):
    import ctypes
    over = dict(precision=1, model_mode=capi.MODEL_GP_ZONE, zero_mode_enabled=0, elastic_residual_tolerance=1e-8,
                elastic_fail_on_nonconvergence=0)
    over.update(kw)
    return params_for(capi, "c2.params", n=n, **over), ctypes


@pytest.mark.gpu
def test_training_pair_inputs_and_target(capi):
    import torch
    from cuda_sto_pf_gb300.solver import Solver
    n = 32
    p, _ = _params(capi, n)
    phi, xB, eta = _micro(n, 5)
    N = n ** 3
    a = torch.empty((8, N), device="cuda")
    t = torch.empty((3, N), device="cuda")
    with Solver(p) as s:
        s.load(phi, xB, eta)
        st = s.training_pair(a, t)
        s.sync()
        assert st.elastic_converged == 1 and st.elastic_iterations >= 2 and st.elastic_warm_start_used == 0
        f = s.fields()
        a_h = a.cpu().numpy()
        assert np.array_equal(a_h[0], f["phi"].astype(np.float32).ravel())
        assert np.array_equal(a_h[1], f["eta"].astype(np.float32).ravel())
        assert np.abs(a_h[2:]).max() > 1e-3                     # eigenstrain present
        t_het = t.cpu().numpy()
        u = s.displacement_k()
    assert np.abs(t_het).max() > 0
    # homogeneous stiffness (S_p = 0): the converged u is u_hom, no correction
    p0, _ = _params(capi, n, S_p=[0.0] * 21)
    with Solver(p0) as s:
        s.load(phi, xB, eta)
        s.training_pair(a, t)
        s.sync()
        t0 = t.cpu().numpy()
    assert np.abs(t0).max() <= 1e-5 * np.abs(t_het).max()
    assert np.isfinite(u).all()


@pytest.mark.gpu
def test_model_start_reaches_the_same_fields(capi):
    """A start from an untrained model, from a zero model and the cold
    start all converge to the tolerance: the fields agree."""
    from cuda_sto_pf_gb300.fno import WarmStartModel
    from cuda_sto_pf_gb300.solver import Solver
    n = 32
    phi, xB, eta = _micro(n, 6)
    out = {}
    for src, kind in ((3, None), (2, "random"), (2, "zero")):
        p, _ = _params(capi, n, elastic_warm_start_source=src)
        with Solver(p) as s:
            model = None
            if kind:
                model = WarmStartModel((n, n, n), modes=4, layers=2, out_scale=[1e-2] * 3)
                if kind == "zero":
                    model.set_params(np.zeros(model.num_params, dtype=np.float32))
                s.set_warm_start_model(model)
            s.load(phi, xB, eta)
            its = []
            for _ in range(2):
                st = s.step(1)
                assert st.elastic_converged == 1
                assert st.elastic_warm_start_used == (2 if kind else 0)
                its.append(st.elastic_iterations)
            out[(src, kind)] = (s.fields(), its)
            s.set_warm_start_model(None)
            if model is not None:
                model.close()
    cold, its_cold = out[(3, None)]
    for key in ((2, "random"), (2, "zero")):
        f, its = out[key]
        for k in ("phi", "xB", "eta"):
            assert rel_l2(f[k], cold[k]) <= 2e-6, (key, k)
    # a zero prediction is the cold start
    assert abs(out[(2, "zero")][1][0] - its_cold[0]) <= 1


@pytest.mark.gpu
def test_model_source_without_model_is_refused(capi):
    from cuda_sto_pf_gb300.fno import WarmStartModel
    from cuda_sto_pf_gb300.solver import Solver
    n = 16
    phi, xB, eta = _micro(n, 7, count=1)
    p, _ = _params(capi, n, elastic_warm_start_source=2)
    with Solver(p) as s:
        s.load(phi, xB, eta)
        with pytest.raises(capi.PfgbError):
            s.step(1)
        with WarmStartModel((8, 8, 8), modes=2, layers=1) as wrong:
            with pytest.raises(capi.PfgbError):
                s.set_warm_start_model(wrong)
    p4, _ = _params(capi, n, elastic_warm_start_source=4)
    with pytest.raises(capi.PfgbError):
        Solver(p4)


@pytest.mark.gpu
def test_trained_model_cuts_cold_iterations(capi):
    """Fit the model on pairs from the solver's own cold solves, then start
    held-out microstructures from its prediction: fewer iterations than the
    cold start, to the same tolerance."""
    import torch
    from cuda_sto_pf_gb300 import fno
    from cuda_sto_pf_gb300.solver import Solver
    n, P = 32, 24
    N = n ** 3
    p, _ = _params(capi, n)
    micro = [_micro(n, 100 + i, count=2 + i % 5) for i in range(P + 4)]
    a = torch.empty((P, 8, N), device="cuda")
    t = torch.empty((P, 3, N), device="cuda")
    with Solver(p) as s:
        fno.make_pairs(s, micro[:P], a, t)
        s.sync()
    in_scale, out_scale = fno.channel_scales(a, t)
    model = fno.WarmStartModel((n, n, n), modes=8, layers=4, in_scale=in_scale, out_scale=out_scale)
    losses = fno.train(model, a, t, steps=300, lr=2e-3)
    assert np.mean(losses[-24:]) < 0.5 * np.mean(losses[:24])
    res = {}
    for src in (3, 2):
        p2, _ = _params(capi, n, elastic_warm_start_source=src)
        its = []
        with Solver(p2) as s:
            s.set_warm_start_model(model)
            for phi, xB, eta in micro[P:]:
                s.load(phi, xB, eta)
                st = s.step(1)
                assert st.elastic_converged == 1
                its.append(st.elastic_iterations)
            s.set_warm_start_model(None)
        res[src] = its
    model.close()
    assert np.mean(res[2]) < np.mean(res[3]), res
