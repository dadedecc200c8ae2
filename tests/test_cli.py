"""The main_cuda driver: invocation, parameter file, raw-field input and the
Results/ layout of the reference's dynamics runs (main_cuda.cu main())."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, params_for


def _exe(capi):
    from cuda_sto_pf_gb300 import build
    return build.EXE


def _run(capi, args, cwd, env=None):
    e = dict(os.environ)
    if env:
        e.update(env)
    return subprocess.run([_exe(capi), *args], cwd=cwd, env=e, capture_output=True, text=True, timeout=600)


def test_cli_requires_param_file(capi, tmp_path):
    r = _run(capi, ["16", "16", "16", "0.01", "2", "1", "1", "1"], tmp_path)
    assert r.returncode == 2
    assert "--pf-param-file" in r.stderr


def test_cli_help(capi, tmp_path):
    r = _run(capi, ["--help"], tmp_path)
    assert r.returncode == 0 and "Nx Ny Nz dt nsteps out_every csv_out_every" in r.stdout


def test_cli_rejects_bad_inputs(capi, tmp_path):
    pf = os.path.join(GOLDEN, "c1.params")
    # unknown mode
    r = _run(capi, ["16", "16", "16", "0.01", "2", "1", "1", "1", "--pf-param-file", pf, "--mode=relax"], tmp_path)
    assert r.returncode == 2 and "--mode=relax" in r.stderr
    # raw_fields without the files, an unknown init mode
    r = _run(capi, ["16", "16", "16", "0.01", "2", "1", "1", "1", "--pf-param-file", pf, "--init-mode", "raw_fields"],
             tmp_path)
    assert r.returncode == 2 and "raw_fields needs" in r.stderr
    r = _run(capi, ["16", "16", "16", "0.01", "2", "1", "1", "1", "--pf-param-file", pf, "--init-mode", "vtk"],
             tmp_path)
    assert r.returncode == 2 and "unknown --init-mode" in r.stderr
    r = _run(capi, ["16", "16", "16", "0.01", "2", "1", "1", "1", "--pf-param-file", pf, "--init-shape", "cube"],
             tmp_path)
    assert r.returncode == 2 and "--init-shape" in r.stderr
    # raw field of the wrong size
    bad = tmp_path / "phi.raw"
    np.zeros(10).tofile(bad)
    r = _run(capi, ["16", "16", "16", "0.01", "2", "1", "1", "1", "--pf-param-file", pf, "--init-mode", "raw_fields",
                    "--init-phi-raw", str(bad), "--init-xB-raw", str(bad)], tmp_path)
    assert r.returncode == 2 and "expected" in r.stderr
    # a model start without a model file
    r = _run(capi, ["16", "16", "16", "0.01", "2", "1", "1", "1", "--pf-param-file", pf,
                    "--elastic-warm-start-source", "2"], tmp_path)
    assert r.returncode == 2 and "--elastic-warm-start-model" in r.stderr
    # checkpoints need the zero mode and a path
    r = _run(capi, ["16", "16", "16", "0.01", "2", "1", "1", "1", "--pf-param-file", pf,
                    "--pf-checkpoint-every", "1", "--pf-checkpoint-path", "x.ckpt"], tmp_path)
    assert r.returncode == 2 and "PF_CONSERVED_Y_ZERO_MODE_V1" in r.stderr
    r = _run(capi, ["16", "16", "16", "0.01", "2", "1", "1", "1", "--pf-param-file", pf,
                    "--pf-zero-mode", "PF_CONSERVED_Y_ZERO_MODE_V1", "--pf-checkpoint-every", "1"], tmp_path)
    assert r.returncode == 2 and "--pf-checkpoint-path" in r.stderr
    # a Y update mode that does not exist
    r = _run(capi, ["16", "16", "16", "0.01", "2", "1", "1", "1", "--pf-param-file", pf,
                    "--pf_y_update_mode", "q_transport"], tmp_path)
    assert r.returncode == 2 and "pf_y_update_mode" in r.stderr
    # malformed parameter file
    pbad = tmp_path / "bad.params"
    pbad.write_text(open(pf).read() + "\nW=abc\n")
    r = _run(capi, ["16", "16", "16", "0.01", "2", "1", "1", "1", "--pf-param-file", str(pbad)], tmp_path)
    assert r.returncode == 2


def _vtk_values(path, shape):
    with open(path) as f:
        lines = f.read().split("\n")
    assert lines[0] == "# vtk DataFile Version 3.0" and lines[3] == "DATASET STRUCTURED_POINTS"
    assert lines[4] == "DIMENSIONS %d %d %d" % shape
    data = np.array(" ".join(lines[10:]).split(), dtype=np.float64)
    nx, ny, nz = shape
    # z outermost, x innermost
    return data.reshape(nz, ny, nx).transpose(2, 1, 0)


@pytest.mark.gpu
def test_cli_dynamics_run_matches_library(capi, tmp_path):
    from cuda_sto_pf_gb300 import workloads
    from cuda_sto_pf_gb300.solver import Solver
    n, steps = 16, 4
    w = workloads.single_sphere(n=n, radius=5.0)
    phi, xB = w["phi"], w["xB"]
    phi.tofile(tmp_path / "phi.raw")
    xB.tofile(tmp_path / "xB.raw")
    pf = os.path.join(GOLDEN, "c2.params")
    r = _run(capi, [str(n), str(n), str(n), "0.01", str(steps), "2", "1", "1", "--pf-param-file", pf,
                    "--init-mode", "raw_fields", "--init-phi-raw", str(tmp_path / "phi.raw"),
                    "--init-xB-raw", str(tmp_path / "xB.raw"), "--pf-zero-mode", "PF_CONSERVED_Y_ZERO_MODE_V1"],
             tmp_path, env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / "R")})
    assert r.returncode == 0, r.stderr
    runs = os.listdir(tmp_path / "R")
    assert len(runs) == 1 and runs[0].startswith("chel_T") and "_cuda_16x16x16_dt0.01_steps4_xB0.030" in runs[0]
    case = tmp_path / "R" / runs[0] / "raw_fields_relax"
    for f in ("pf_input.params", "vf_precip_vs_time_raw_fields_relax.csv", "elastic_solver_trace.csv",
              "pf_zero_mode_trace.csv", "performance_summary.json", "summary.txt", "phi_init.vtk", "phi_2.vtk",
              "phi_4.vtk", "xB_0.vtk", "xBtot_0.vtk", "xBtot_4.vtk"):
        assert (case / f).exists(), f
    # dynamics writes no *_final files (main_cuda.cu:33815-33840: only a last
    # step off the out_every schedule gets its own set)
    assert not any("_final" in f for f in os.listdir(case))
    rows = (case / "vf_precip_vs_time_raw_fields_relax.csv").read_text().strip().split("\n")
    assert rows[0] == "step,t_code,t_real_s,vf_precip,R_avg" and len(rows) == steps + 2
    assert len((case / "elastic_solver_trace.csv").read_text().strip().split("\n")) == steps + 1
    # the same run through the library API
    p = params_for(capi, "c2.params", n=n, zero_mode_enabled=1, precision=0)
    import ctypes
    capi.load().pfgb_prepare_raw_fields(ctypes.byref(p), 0.07, phi.ctypes.data, xB.ctypes.data, None, None,
                                        phi.size)
    with Solver(p) as s:
        s.load(phi, xB)
        s.step(steps)
        f = s.fields()
        d = s.diagnostics()
    last = rows[-1].split(",")
    assert int(last[0]) == steps
    assert abs(float(last[3]) - d.vf_precip) <= 1e-7 * max(1e-12, d.vf_precip)
    got = _vtk_values(case / "phi_4.vtk", (n, n, n))
    assert np.abs(got - f["phi"]).max() <= 6e-6


@pytest.mark.gpu
def test_cli_minimize_run(capi, tmp_path):
    from cuda_sto_pf_gb300 import workloads
    n, iters = 16, 5
    w = workloads.single_sphere(n=n, radius=5.0)
    w["phi"].tofile(tmp_path / "phi.raw")
    w["xB"].tofile(tmp_path / "xB.raw")
    pf = os.path.join(GOLDEN, "c2.params")
    r = _run(capi, [str(n), str(n), str(n), "0.05", "100", "50", "1", "1", "--pf-param-file", pf,
                    "--mode=minimize", "--minimize-full-model", "--minimize-max-iter", str(iters),
                    "--minimize-dt", "0.05", "--V0", "0.05", "--init-mode", "raw_fields",
                    "--init-phi-raw", str(tmp_path / "phi.raw"), "--init-xB-raw", str(tmp_path / "xB.raw")],
             tmp_path, env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / "R")})
    assert r.returncode == 0, r.stderr
    runs = os.listdir(tmp_path / "R")
    assert len(runs) == 1 and "_steps5_r" in runs[0] and runs[0].endswith("nm_xB0.030")
    case = tmp_path / "R" / runs[0] / "raw_fields_relax"
    energy = [f for f in os.listdir(case) if f.startswith("energy_minimize_T")]
    assert len(energy) == 1 and energy[0].endswith("_raw_fields_relax.csv")
    rows = (case / energy[0]).read_text().strip().split("\n")
    assert rows[0].startswith("iter,dt,mean_h,V0,lambda,F_surf_hat") and len(rows) == iters + 1
    last = rows[-1].split(",")
    assert int(last[0]) == iters and abs(float(last[3]) - 0.05) < 1e-12
    assert abs(float(last[2]) - 0.05) < 1e-3          # <h> held at V0
    for f in ("phi_init_raw_fields_relax.vtk", "xB_init_raw_fields_relax.vtk", "phi_final_raw_fields_relax.vtk",
              "xB_final_raw_fields_relax.vtk", "vf_precip_vs_time_raw_fields_relax.csv", "elastic_solver_trace.csv"):
        assert (case / f).exists(), f


@pytest.mark.gpu
def test_cli_learned_start(capi, tmp_path):
    """--elastic-warm-start-model: the trace marks model-started solves (2)."""
    from cuda_sto_pf_gb300 import workloads
    from cuda_sto_pf_gb300.fno import WarmStartModel
    n, steps = 16, 3
    w = workloads.single_sphere(n=n, radius=5.0)
    w["phi"].tofile(tmp_path / "phi.raw")
    w["xB"].tofile(tmp_path / "xB.raw")
    with WarmStartModel((n, n, n), modes=4, layers=2, out_scale=[1e-3] * 3) as m:
        m.save(str(tmp_path / "start.pfgbfno"))
    pf = os.path.join(GOLDEN, "c2.params")
    r = _run(capi, [str(n), str(n), str(n), "0.01", str(steps), "10", "1", "1", "--pf-param-file", pf,
                    "--init-mode", "raw_fields", "--init-phi-raw", str(tmp_path / "phi.raw"),
                    "--init-xB-raw", str(tmp_path / "xB.raw"), "--precision", "fp32",
                    "--elastic-warm-start-model", str(tmp_path / "start.pfgbfno"),
                    "--elastic-warm-start-source", "2"],
             tmp_path, env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / "R")})
    assert r.returncode == 0, r.stderr
    run = os.listdir(tmp_path / "R")[0]
    rows = (tmp_path / "R" / run / "raw_fields_relax" / "elastic_solver_trace.csv").read_text().strip().split("\n")
    assert len(rows) == steps + 1
    assert all(row.split(",")[1] == "2" for row in rows[1:])


@pytest.mark.gpu
def test_cli_checkpoint_restart(capi, tmp_path):
    """--pf-checkpoint-every / --pf-restart-from: two steps, a checkpoint,
    a restarted run to step 4; its final checkpoint holds the same fields
    as an uninterrupted 4-step run's."""
    import ctypes
    from cuda_sto_pf_gb300 import workloads
    n = 16
    w = workloads.single_sphere(n=n, radius=5.0)
    w["phi"].tofile(tmp_path / "phi.raw")
    w["xB"].tofile(tmp_path / "xB.raw")
    pf = os.path.join(GOLDEN, "c2.params")
    base = [str(n), str(n), str(n), "0.01", "STEPS", "10", "1", "1", "--pf-param-file", pf, "--init-mode",
            "raw_fields", "--init-phi-raw", str(tmp_path / "phi.raw"), "--init-xB-raw", str(tmp_path / "xB.raw"),
            "--pf-zero-mode", "PF_CONSERVED_Y_ZERO_MODE_V1", "--pf-initial-state-class", "SPHERE_16"]

    def run(steps, root, extra):
        args = [steps if a == "STEPS" else a for a in base] + extra
        r = _run(capi, args, tmp_path, env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / root)})
        assert r.returncode == 0, r.stderr
        return r

    run("2", "A", ["--pf-checkpoint-every", "2", "--pf-checkpoint-path", str(tmp_path / "s2.ckpt")])
    r = run("4", "B", ["--pf-restart-from", str(tmp_path / "s2.ckpt"), "--pf-checkpoint-every", "4",
                       "--pf-checkpoint-path", str(tmp_path / "b4.ckpt")])
    assert "accepted_step=2" in r.stdout
    run("4", "C", ["--pf-checkpoint-every", "4", "--pf-checkpoint-path", str(tmp_path / "c4.ckpt")])
    # a restart with another identity is refused
    args = [("4" if a == "STEPS" else a) for a in base] + ["--pf-restart-from", str(tmp_path / "s2.ckpt")]
    args[args.index("SPHERE_16")] = "OTHER"
    r = _run(capi, args, tmp_path, env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / "D")})
    assert r.returncode == 2 and "rejected" in r.stderr
    lib = capi.load()
    p = params_for(capi, "c2.params", n=n, zero_mode_enabled=1)
    out = {}
    for tag in ("b4", "c4"):
        st = capi.CkptState()
        st.nx = st.ny = st.nz = n
        buf = {k: np.zeros(n ** 3) for k in ("phi", "Y", "xB", "dY")}
        u = np.zeros(6 * n * n * (n // 2 + 1), dtype=np.float32)
        st.phi, st.Y, st.xB, st.dY_dt_prev = (buf[k].ctypes.data for k in ("phi", "Y", "xB", "dY"))
        st.displacement_k = u.ctypes.data
        prov = capi.CkptProvenance()
        capi.check(lib.pfgb_checkpoint_provenance_for(ctypes.byref(p), b"SPHERE_16", None, None, ctypes.byref(prov)),
                   "provenance")
        capi.check(lib.pfgb_checkpoint_read_file(str(tmp_path / (tag + ".ckpt")).encode(), ctypes.byref(prov),
                                                 ctypes.byref(st)), "read " + tag)
        assert st.accepted_step == 4 and st.elastic_source_field_step == 3
        out[tag] = buf
    for k in ("phi", "Y", "xB", "dY"):
        assert np.abs(out["b4"][k] - out["c4"][k]).max() <= 1e-12 * max(1.0, np.abs(out["c4"][k]).max()), k


@pytest.mark.gpu
def test_cli_output_formats(capi, tmp_path):
    """--output-format vtk-binary / raw beside the default ASCII VTK, and the
    reference's CUDA_STO_SUPPRESS_VTK_OUTPUT switch."""
    from cuda_sto_pf_gb300 import workloads
    n = 16
    w = workloads.single_sphere(n=n, radius=5.0)
    w["phi"].tofile(tmp_path / "phi.raw")
    w["xB"].tofile(tmp_path / "xB.raw")
    pf = os.path.join(GOLDEN, "c2.params")
    base = [str(n), str(n), str(n), "0.01", "2", "10", "1", "1", "--pf-param-file", pf, "--init-mode", "raw_fields",
            "--init-phi-raw", str(tmp_path / "phi.raw"), "--init-xB-raw", str(tmp_path / "xB.raw")]
    dirs = {}
    for fmt in ("vtk", "vtk-binary", "raw"):
        r = _run(capi, base + ["--output-format", fmt], tmp_path, env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / fmt)})
        assert r.returncode == 0, r.stderr
        run = os.listdir(tmp_path / fmt)[0]
        dirs[fmt] = tmp_path / fmt / run / "raw_fields_relax"
    # 2 steps with out_every 10: the last step is written as output number
    # 2 // 10 + 1 = 1 (main_cuda.cu:33815-33840)
    raw = np.fromfile(dirs["raw"] / "phi_1.raw", dtype=np.float64).reshape(n, n, n)
    blob = (dirs["vtk-binary"] / "phi_1.vtk").read_bytes()
    head = b"LOOKUP_TABLE default\n"
    data = np.frombuffer(blob[blob.index(head) + len(head):][:8 * n ** 3], dtype=">f8")
    assert blob[blob.index(b"Simulation\n") + 11:].startswith(b"BINARY\n")
    assert np.array_equal(data.reshape(n, n, n).transpose(2, 1, 0), raw)   # z outer, x inner
    asc = _vtk_values(dirs["vtk"] / "phi_1.vtk", (n, n, n))
    assert np.abs(asc - raw).max() <= 5.1e-6
    assert (dirs["raw"] / "xBtot_1.raw").exists() and not (dirs["raw"] / "phi_1.vtk").exists()
    r = _run(capi, base, tmp_path, env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / "S"), "CUDA_STO_SUPPRESS_VTK_OUTPUT": "1"})
    assert r.returncode == 0 and "VTK_OUTPUT_SUPPRESSED field=phi" in r.stdout
    run = os.listdir(tmp_path / "S")[0]
    assert not any(f.endswith(".vtk") for f in os.listdir(tmp_path / "S" / run / "raw_fields_relax"))


@pytest.mark.gpu
def test_cli_seeded_initialisation(capi, tmp_path):
    """Without raw fields the run starts from the seeded initialiser
    (initialize_fields_cuda): case directory named after the shape, and the
    initial phi equal to the restatement in oracle/init_oracle.py."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(GOLDEN), "..", "oracle"))
    import init_oracle
    n = 24
    pf = os.path.join(GOLDEN, "c2.params")
    r = _run(capi, [str(n), str(n), str(n), "0.01", "1", "10", "1", "1", "--pf-param-file", pf, "--radius", "6",
                    "--init-shape", "ellipsoid", "--init-axis-ratio-rz", "0.5", "--init-tilt-theta-deg", "30",
                    "--init-phi-noise-amp", "0.01", "--seed", "99"],
             tmp_path, env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / "R")})
    assert r.returncode == 0, r.stderr
    run = os.listdir(tmp_path / "R")[0]
    case = tmp_path / "R" / run / "case_test-1_ellipsoid_th30_ph0_noise1e-02"
    assert case.is_dir(), os.listdir(tmp_path / "R" / run)
    p = params_for(capi, "c2.params", n=n, ic_phi_seed_radius=6.0, init_shape_mode=1, init_axis_ratio_rz=0.5,
                   init_tilt_theta_deg=30.0, init_use_rotation=1, init_phi_noise_amp=0.01, seed=99)
    want, _ = init_oracle.seed_fields(p)
    got = _vtk_values(case / "phi_init.vtk", (n, n, n))
    assert np.abs(got - want).max() <= 5.1e-6


@pytest.mark.gpu
def test_cli_vtk_continuation(capi, tmp_path):
    """--mode=dynamics-continue / --mode=minimize-continue with
    --continue-phi-vtk [--continue-xB-vtk] (main_cuda.cu:22752-22770,
    2602-2650, 25363-25480): the fields come from the source run's ASCII
    VTK files, the outputs go to a new case directory continue_dyn_<n> /
    continue_min_<n> under the source run's root (re-rooted under
    CUDA_STO_RESULTS_ROOT), the CSVs keep the source case's tag and a
    continuation writes no step-0 row."""
    import ctypes
    from cuda_sto_pf_gb300 import workloads
    from cuda_sto_pf_gb300.solver import Solver
    n = 16
    w = workloads.single_sphere(n=n, radius=5.0)
    w["phi"].tofile(tmp_path / "phi.raw")
    w["xB"].tofile(tmp_path / "xB.raw")
    pf = os.path.join(GOLDEN, "c2.params")
    raw = ["--init-mode", "raw_fields", "--init-phi-raw", str(tmp_path / "phi.raw"), "--init-xB-raw",
           str(tmp_path / "xB.raw")]
    # dynamics: 4 steps, then 3 more from the step-4 VTK files
    r = _run(capi, [str(n)] * 3 + ["0.01", "4", "4", "1", "1", "--pf-param-file", pf] + raw, tmp_path,
             env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / "A")})
    assert r.returncode == 0, r.stderr
    run = os.listdir(tmp_path / "A")[0]
    src = tmp_path / "A" / run / "raw_fields_relax"
    r = _run(capi, [str(n)] * 3 + ["0.01", "3", "3", "1", "1", "--pf-param-file", pf, "--mode=dynamics-continue",
                                   "--continue-phi-vtk", str(src / "phi_4.vtk"), "--continue-xB-vtk",
                                   str(src / "xB_4.vtk")], tmp_path, env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / "B")})
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    case = tmp_path / "B" / run / "continue_dyn_1"
    assert (case / "phi_3.vtk").exists() and (case / "pf_input.params").exists()
    rows = (case / "vf_precip_vs_time_raw_fields_relax.csv").read_text().strip().split("\n")
    assert rows[0] == "step,t_code,t_real_s,vf_precip,R_avg" and [int(x.split(",")[0]) for x in rows[1:]] == [1, 2, 3]
    # the same continuation through the library from the VTK values
    phi0 = _vtk_values(src / "phi_4.vtk", (n, n, n))
    xB0 = _vtk_values(src / "xB_4.vtk", (n, n, n))
    p = params_for(capi, "c2.params", n=n, precision=0)
    capi.load().pfgb_prepare_raw_fields(ctypes.byref(p), float("nan"), phi0.ctypes.data, xB0.ctypes.data, None, None,
                                        phi0.size)
    with Solver(p) as s:
        s.load(phi0, xB0)
        s.step(3)
        f = s.fields()
    assert np.abs(_vtk_values(case / "phi_3.vtk", (n, n, n)) - f["phi"]).max() <= 6e-6
    # a second continuation from inside the first takes the next index
    r = _run(capi, [str(n)] * 3 + ["0.01", "2", "2", "1", "1", "--pf-param-file", pf, "--mode=dynamics-continue",
                                   "--continue-phi-vtk", str(case / "phi_3.vtk")], tmp_path,
             env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / "B")})
    assert r.returncode == 0, r.stderr[-2000:]
    assert (tmp_path / "B" / run / "continue_dyn_2" / "phi_2.vtk").exists()
    # full-model minimize, then minimize-continue from its final files
    mz = ["--mode=minimize", "--minimize-full-model", "--minimize-max-iter", "3", "--minimize-dt", "0.05", "--V0", "0.05"]
    r = _run(capi, [str(n)] * 3 + ["0.05", "100", "50", "1", "1", "--pf-param-file", pf] + mz + raw, tmp_path,
             env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / "C")})
    assert r.returncode == 0, r.stderr
    run = os.listdir(tmp_path / "C")[0]
    src = tmp_path / "C" / run / "raw_fields_relax"
    r = _run(capi, [str(n)] * 3 + ["0.05", "100", "50", "1", "1", "--pf-param-file", pf, "--mode=minimize-continue",
                                   "--minimize-full-model", "--minimize-max-iter", "2", "--minimize-dt", "0.05",
                                   "--V0", "0.05", "--continue-phi-vtk", str(src / "phi_final_raw_fields_relax.vtk"),
                                   "--continue-xB-vtk", str(src / "xB_final_raw_fields_relax.vtk")], tmp_path,
             env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / "D")})
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    case = tmp_path / "D" / run / "continue_min_1"
    names = os.listdir(case)
    assert "phi_final_continue_min_1.vtk" in names and "xB_final_continue_min_1.vtk" in names, names
    energy = [x for x in names if x.startswith("energy_minimize_") and x.endswith("_raw_fields_relax.csv")]
    assert len(energy) == 1, names
    assert len((case / energy[0]).read_text().strip().split("\n")) == 3
    # continuation refusals
    r = _run(capi, [str(n)] * 3 + ["0.05", "10", "5", "1", "1", "--pf-param-file", pf, "--mode=minimize-continue"],
             tmp_path)
    assert r.returncode == 2 and "--continue-phi-vtk" in r.stderr
    r = _run(capi, [str(n)] * 3 + ["0.01", "2", "2", "1", "1", "--pf-param-file", pf, "--continue-phi-vtk",
                                   str(src / "phi_final_raw_fields_relax.vtk")] + raw, tmp_path)
    assert r.returncode == 2 and "cannot be combined" in r.stderr


@pytest.mark.gpu
def test_cli_phi_only_minimize(capi, tmp_path):
    """--mode=minimize without --minimize-full-model: the reference's default
    phi-only minimize from the seeded phi (raw fields are refused there),
    no vf CSV, phi files only."""
    n = 16
    pf = os.path.join(GOLDEN, "c2.params")
    r = _run(capi, [str(n)] * 3 + ["0.05", "100", "50", "1", "1", "--pf-param-file", pf, "--mode=minimize",
                                   "--minimize-max-iter", "4", "--radius", "5", "--V0", "0.05"], tmp_path,
             env={"CUDA_STO_RESULTS_ROOT": str(tmp_path / "R")})
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    run = os.listdir(tmp_path / "R")[0]
    case = tmp_path / "R" / run / os.listdir(tmp_path / "R" / run)[0]
    names = os.listdir(case)
    assert not any(x.startswith("vf_precip_vs_time") for x in names), names
    assert any(x.startswith("phi_final_") for x in names) and not any(x.startswith("xB_final_") for x in names)
    energy = [x for x in names if x.startswith("energy_minimize_")][0]
    rows = (case / energy).read_text().strip().split("\n")
    assert len(rows) == 5 and rows[1].split(",")[7] == "nan"   # F_chem_excess_hat is NaN
    w = np.ones((n, n, n)).tofile(tmp_path / "phi.raw")
    r = _run(capi, [str(n)] * 3 + ["0.05", "100", "50", "1", "1", "--pf-param-file", pf, "--mode=minimize",
                                   "--init-mode", "raw_fields", "--init-phi-raw", str(tmp_path / "phi.raw"),
                                   "--init-xB-raw", str(tmp_path / "phi.raw")], tmp_path)
    assert r.returncode == 2 and "full-model minimize" in r.stderr
