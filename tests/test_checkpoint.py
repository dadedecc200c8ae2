"""Zero-mode checkpoints in the reference's file format
(pf_zero_mode_checkpoint.{h,cpp}; main_cuda.cu:27340-28100 restart,
33494-33560 write).

The library's writer and reader are pinned against the reference's own
writer and reader, compiled from the reference tree into
oracle/_ref/libpfckpt.so (oracle/build_oracle.py --ref): the same state
gives byte-identical V3 and V4 files, and each side reads the other's
files.  The provenance fingerprints are restated here from their
definition (main_cuda.cu:4187-4264).  The GPU test checks that a run
restored from a checkpoint continues like the uninterrupted run."""
import ctypes
import os
import struct
import sys

import numpy as np
import pytest

from conftest import REPO, params_for, rel_l2

REF_CKPT = os.path.join(REPO, "oracle", "_ref", "libpfckpt.so")


def _ref():
    if not os.path.exists(REF_CKPT):
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import build_oracle
        if build_oracle.build_ref_checkpoint() is None:
            pytest.skip("reference checkpoint code not available (reference tree absent)")
    from cuda_sto_pf_gb300 import capi
    L = ctypes.CDLL(REF_CKPT)
    L.ref_ckpt_write.restype = ctypes.c_int
    L.ref_ckpt_write.argtypes = [ctypes.c_char_p, ctypes.POINTER(capi.CkptState), ctypes.c_char_p, ctypes.c_int]
    L.ref_ckpt_read.restype = ctypes.c_int
    L.ref_ckpt_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(capi.CkptProvenance), ctypes.POINTER(capi.CkptState),
                                ctypes.c_char_p, ctypes.c_int]
    return L


def _fnv(data: bytes, h=1469598103934665603):
    for b in data:
        h ^= b
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def _param_fp(p):
    d = struct.pack("<3i", p.Nx, p.Ny, p.Nz)
    for v in (p.dt, p.temperature_C, p.dx, p.dy, p.dz, p.v_A, p.v_B, p.D_alpha, p.D_compound, p.L_phi,
              p.kappa_phi, p.W, p.Y_clip, p.xB_eps):
        d += struct.pack("<d", v)
    d += struct.pack("<2i", p.enable_Y_rhs_previous_time_level, p.disable_Y_rhs_gamma_term)
    ymode = ["lagged_rhs", "storage_exact", "x_transport_projection_split"][p.pf_y_update_mode]
    for s in ("legacy", ymode, "SM_EXPLICIT_CONTEXT_N_V1", "SM_TANGENT_N_V1"):
        d += s.encode() + b"\0"
    h = _fnv(d)
    return h or 1


def _elastic_fp(p):
    d = struct.pack("<3i", p.Nx, p.Ny, p.Nz) + struct.pack("<3d", p.dx, p.dy, p.dz)
    d += struct.pack("<5i", p.elastic_enabled, p.elastic_warm_start_enabled, p.elastic_residual_control_enabled,
                     p.elastic_iter_min, p.elastic_iter_max)
    d += struct.pack("<2d", p.elastic_residual_tolerance, p.elastic_residual_absolute_floor)
    d += struct.pack("<i", p.elastic_fail_on_nonconvergence)
    d += struct.pack("<42d", *(list(p.S) + list(p.S_p)))
    d += struct.pack("<13d", *(list(p.eps00) + [p.eps_iso_over_vB] + list(p.E0)))
    return _fnv(d) or 1


@pytest.mark.parametrize("name", ["c1.params", "c2.params"])
def test_fingerprints_match_their_definition(capi, name):
    lib = capi.load()
    p = params_for(capi, name, n=24)
    assert lib.pfgb_parameter_fingerprint(ctypes.byref(p)) == _param_fp(p)
    assert lib.pfgb_elastic_solver_fingerprint(ctypes.byref(p)) == _elastic_fp(p)
    assert lib.pfgb_fnv1a64(b"abc", 3, 1469598103934665603) == _fnv(b"abc")
    q = params_for(capi, name, n=24, pf_y_update_mode=capi.Y_STORAGE_EXACT)
    assert lib.pfgb_parameter_fingerprint(ctypes.byref(q)) == _param_fp(q) != _param_fp(p)


class _State:
    """A random checkpoint state with its own host buffers."""

    def __init__(self, capi, shape=(6, 5, 8), elastic=True, seed=1, step=7, identity=None):
        rng = np.random.default_rng(seed)
        self.p = params_for(capi, "c2.params", n=shape[0])
        self.p.Nx, self.p.Ny, self.p.Nz = shape
        if not elastic:
            self.p.elastic_warm_start_enabled = 0
            self.p.elastic_residual_control_enabled = 0
        N = shape[0] * shape[1] * shape[2]
        Nk = shape[0] * shape[1] * (shape[2] // 2 + 1)
        self.f = {k: rng.standard_normal(N) for k in ("phi", "Y", "xB", "dY")}
        self.u = rng.standard_normal(6 * Nk).astype(np.float32)
        s = capi.CkptState()
        ident = identity or {}
        enc = lambda k: ident[k].encode() if k in ident else None
        capi.check(capi.load().pfgb_checkpoint_provenance_for(
            ctypes.byref(self.p), enc("initial_state_class"), enc("fixture_manifest_sha256"),
            enc("profile_library_manifest_sha256"), ctypes.byref(s.provenance)), "provenance_for")
        s.accepted_step = step
        s.nx, s.ny, s.nz = shape
        s.elastic_present = 1 if elastic else 0
        s.dt_code = self.p.dt
        s.temperature_K = self.p.temperature_C + 273.15
        s.target_mass_code, s.last_lambda = 123.456, -1.5e-4
        s.last_residual_code, s.last_derivative_code = 3e-13, 2.75
        s.last_iterations, s.accepted_zero_mode_steps = 4, step
        if elastic:
            s.elastic_source_field_step, s.elastic_last_iterations = step - 1, 13
            s.elastic_last_relative_residual = 7.5e-9
        s.phi, s.Y, s.xB, s.dY_dt_prev = (self.f[k].ctypes.data for k in ("phi", "Y", "xB", "dY"))
        s.displacement_k = self.u.ctypes.data if elastic else None
        self.s = s
        self.N, self.Nk = N, Nk

    def empty(self, capi):
        out = capi.CkptState()
        out.nx, out.ny, out.nz = self.s.nx, self.s.ny, self.s.nz
        self.o = {k: np.zeros(self.N) for k in ("phi", "Y", "xB", "dY")}
        self.ou = np.zeros(6 * self.Nk, dtype=np.float32)
        out.phi, out.Y, out.xB, out.dY_dt_prev = (self.o[k].ctypes.data for k in ("phi", "Y", "xB", "dY"))
        out.displacement_k = self.ou.ctypes.data
        return out


@pytest.mark.parametrize("elastic", [False, True], ids=["V3", "V4"])
def test_files_match_the_reference_byte_for_byte(capi, tmp_path, elastic):
    ref = _ref()
    st = _State(capi, elastic=elastic, identity={"initial_state_class": "FIXTURE_A",
                                                 "fixture_manifest_sha256": "ab" * 32})
    ours, theirs = str(tmp_path / "ours.ckpt"), str(tmp_path / "ref.ckpt")
    capi.check(capi.load().pfgb_checkpoint_write_file(ours.encode(), ctypes.byref(st.s)), "write")
    err = ctypes.create_string_buffer(256)
    assert ref.ref_ckpt_write(theirs.encode(), ctypes.byref(st.s), err, 256) == 1, err.value
    a, b = open(ours, "rb").read(), open(theirs, "rb").read()
    assert len(a) == (904 if elastic else 800) + 4 * 8 * st.N + (24 * st.Nk if elastic else 0)
    assert a == b
    assert not os.path.exists(ours + ".tmp")


@pytest.mark.parametrize("elastic", [False, True], ids=["V3", "V4"])
def test_each_side_reads_the_other(capi, tmp_path, elastic):
    ref = _ref()
    lib = capi.load()
    st = _State(capi, elastic=elastic, seed=3)
    ours, theirs = str(tmp_path / "ours.ckpt"), str(tmp_path / "ref.ckpt")
    capi.check(lib.pfgb_checkpoint_write_file(ours.encode(), ctypes.byref(st.s)), "write")
    err = ctypes.create_string_buffer(256)
    assert ref.ref_ckpt_write(theirs.encode(), ctypes.byref(st.s), err, 256) == 1
    # the library reads the reference's file
    out = st.empty(capi)
    capi.check(lib.pfgb_checkpoint_read_file(theirs.encode(), ctypes.byref(st.s.provenance), ctypes.byref(out)),
               "read")
    for k in st.f:
        assert np.array_equal(st.o[k], st.f[k])
    if elastic:
        assert np.array_equal(st.ou, st.u)
        assert out.elastic_source_field_step == st.s.elastic_source_field_step
    assert (out.accepted_step, out.last_iterations, out.target_mass_code) == (7, 4, 123.456)
    # the reference reads the library's file
    out2 = st.empty(capi)
    assert ref.ref_ckpt_read(ours.encode(), ctypes.byref(st.s.provenance), ctypes.byref(out2), err, 256) == 1, \
        err.value
    for k in st.f:
        assert np.array_equal(st.o[k], st.f[k])
    v = ctypes.c_int32()
    nx = ctypes.c_int32()
    capi.check(lib.pfgb_checkpoint_peek(ours.encode(), ctypes.byref(v), ctypes.byref(nx), None, None, None), "peek")
    assert (v.value, nx.value) == ((4 if elastic else 3), 6)


def test_rejections(capi, tmp_path):
    ref = _ref()
    lib = capi.load()
    st = _State(capi, elastic=True, seed=5)
    path = str(tmp_path / "a.ckpt")
    capi.check(lib.pfgb_checkpoint_write_file(path.encode(), ctypes.byref(st.s)), "write")
    err = ctypes.create_string_buffer(256)

    def both_reject(p, prov):
        o1 = st.empty(capi)
        r1 = lib.pfgb_checkpoint_read_file(p.encode(), ctypes.byref(prov), ctypes.byref(o1))
        o2 = st.empty(capi)
        r2 = ref.ref_ckpt_read(p.encode(), ctypes.byref(prov), ctypes.byref(o2), err, 256)
        return r1 != 0 and r2 == 0

    # another identity / another fingerprint
    for field, value in (("initial_state_class", b"OTHER"), ("parameter_fingerprint", 12345),
                         ("elastic_solver_fingerprint", 99)):
        prov = capi.CkptProvenance.from_buffer_copy(st.s.provenance)
        setattr(prov, field, value)
        assert both_reject(path, prov), field
    # a flipped payload byte, a truncated file, a trailing byte
    raw = bytearray(open(path, "rb").read())
    for name, data in (("flip", raw[:1000] + bytes([raw[1000] ^ 1]) + raw[1001:]), ("trunc", raw[:-3]),
                       ("trail", raw + b"\0")):
        q = str(tmp_path / (name + ".ckpt"))
        open(q, "wb").write(bytes(data))
        assert both_reject(q, st.s.provenance), name
    # V3 where the elastic warm state is required
    s3 = _State(capi, elastic=False, seed=6)
    q = str(tmp_path / "v3.ckpt")
    capi.check(lib.pfgb_checkpoint_write_file(q.encode(), ctypes.byref(s3.s)), "write")
    assert both_reject(q, st.s.provenance)
    # invalid states are not written
    bad = _State(capi, elastic=True, seed=7)
    bad.s.elastic_source_field_step = 3   # must be accepted_step - 1
    assert lib.pfgb_checkpoint_write_file(str(tmp_path / "b.ckpt").encode(), ctypes.byref(bad.s)) != 0
    bad2 = _State(capi, elastic=False, seed=8)
    bad2.f["phi"][3] = np.nan
    assert lib.pfgb_checkpoint_write_file(str(tmp_path / "c.ckpt").encode(), ctypes.byref(bad2.s)) != 0


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-5)])
def test_restart_continues_the_run(capi, tmp_path, prec, tol):
    """Two steps, checkpoint, restore into a fresh context, two more steps:
    the same fields as four uninterrupted steps (FP64 fields: to 1e-12; FP32
    fields: within the FP32 form's 1e-5 bound, since the restored Y is one
    float instead of the float plus FP64 offset the running context holds)."""
    from cuda_sto_pf_gb300 import workloads
    from cuda_sto_pf_gb300.solver import Solver
    n = 32
    p = params_for(capi, "c2.params", n=n, precision=prec, zero_mode_enabled=1)
    w = workloads.single_sphere(n=n, radius=7.0)
    phi, xB = w["phi"], w["xB"]
    capi.load().pfgb_prepare_raw_fields(ctypes.byref(p), 0.07, phi.ctypes.data, xB.ctypes.data, None, None, phi.size)
    with Solver(p) as s:
        s.load(phi, xB)
        s.step(4)
        want = s.fields()
    path = str(tmp_path / "run.ckpt")
    with Solver(p) as s:
        s.load(phi, xB)
        s.step(2)
        s.checkpoint_save(path, initial_state_class="SPHERE_R7")
    ver = ctypes.c_int32()
    capi.check(capi.load().pfgb_checkpoint_peek(path.encode(), ctypes.byref(ver), None, None, None, None), "peek")
    assert ver.value == 4
    with Solver(p) as s:
        with pytest.raises(capi.PfgbError):   # another identity is another run
            s.checkpoint_restore(path, initial_state_class="OTHER")
        s.checkpoint_restore(path, initial_state_class="SPHERE_R7")
        st = s.step(2)
        assert st.step == 4 and st.elastic_warm_start_used == 1
        got = s.fields()
    for k in ("phi", "xB", "Y", "dYdt"):
        assert rel_l2(got[k], want[k]) <= tol, k

