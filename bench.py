"""Benchmark: dynamics time step of the CUDA_STO_PF hot path on GB300.

Workload (default): 246^3 grid, gp_zone model, 60 ellipsoidal precipitates
(log-normal radii, median 6 cells, sigma_ln 0.3, aspect ratios U[0.5,1],
random rotations, non-overlapping), 20 GP-zone eta sites of radius 3,
heterogeneous elasticity S_p = C_Ag2Te - C_PbTe (cubic 60/25/15 vs
108/7.7/13 GPa), zero mode on, FP32 fields with FP64 reductions and zero mode,
dt = 0.01.  One step = one full dynamics time step (elastic fixed point,
phi / eta Allen-Cahn, Y Cahn-Hilliard, zero-mode mass solve).

Metric: cell-steps/s (N * steps / s, the reference's Mpts/s print).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU: a single case does not shard (every 3D FFT is global); N > 1
runs N independent replicas, one per rank ("replicas only"), with a barrier
and max-over-ranks timing.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "cell-steps/s @246^3 elastic (dynamics step, gp_zone, heterogeneous S_p, zero mode)"
PARAMS = os.path.join(REPO, "tests", "golden", "c2.params")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=246)
    ap.add_argument("--shape", default="", help="Nx,Ny,Nz (profiling cases; default n^3)")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--elastic-tol", type=float, default=1e-8)
    ap.add_argument("--cpu-sample-n", type=int, default=128)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain-fp64", action="store_true")
    ap.add_argument("--no-chebyshev", action="store_true", help="the reference's plain elastic iteration")
    ap.add_argument("--no-extrapolate", action="store_true",
                    help="start each elastic solve from the previous solution (the reference's warm start)")
    ap.add_argument("--extrapolate-order", type=int, default=None, choices=[1, 2, 3, 4, 5],
                    help="order of the extrapolated warm start (default: EXTRAPOLATE)")
    ap.add_argument("--fft-autotune", type=int, default=0, choices=[0, 1, 2, 3],
                    help="bits of the generic engine's tile autotuner (grids whose axes are not 246 long): "
                         "1 the x / y passes, 2 the z passes")
    ap.add_argument("--fft-tensor-cores", type=int, default=None,
                    help="1: the 41-point stage of the elastic y passes on the tensor cores (default: FFT_TENSOR_CORES)")
    ap.add_argument("--profile-json", default="")
    ap.add_argument("--fno-n", type=int, default=128)
    ap.add_argument("--fno-base", type=int, default=128, help="distinct generated microstructures")
    ap.add_argument("--fno-pairs", type=int, default=1024, help="training pairs (base x cube symmetries)")
    ap.add_argument("--fno-train-steps", type=int, default=6000)
    ap.add_argument("--fno-eval-steps", type=int, default=300)
    ap.add_argument("--particles", type=int, default=None,
                    help="precipitate count (default: 60 scaled by the grid volume over 246^3)")
    ap.add_argument("--median-radius", type=float, default=6.0, help="median precipitate radius in cells")
    ap.add_argument("--eta-sites", type=int, default=None,
                    help="GP-zone eta sites (default: 20 scaled by the grid volume over 246^3)")
    ap.add_argument("--horizon-chosen", default="fp32", choices=["fp32", "fp64", "fp64-plain"],
                    help="horizon workload: the arm compared with the plain FP64 form")
    ap.add_argument("--horizon-plain-tol", type=float, default=None,
                    help="horizon workload: elastic tolerance of the plain FP64 arm (default --elastic-tol)")
    ap.add_argument("--horizon-marks", default="8,25,50,100",
                    help="horizon workload: step counts at which the fields are compared")
    ap.add_argument("--workload", default="c2", choices=["c2", "sweep", "fno", "fno-step", "horizon"],
                    help="c2: the 246^3 dynamics step (default); sweep: the batched minimize sweep")
    ap.add_argument("--sweep-cases", type=int, default=48)
    ap.add_argument("--sweep-iters", type=int, default=500)
    ap.add_argument("--sweep-concurrency", type=int, default=8)
    ap.add_argument("--sweep-autotune", type=int, default=0, choices=[0, 1, 2, 3],
                    help="tile autotuner of the generic engine (fft_autotune) in the sweep; the rule's tiles are "
                         "within 3%% of the tuned ones under the sweep's sharing, and tuning costs about 4 s")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# elastic iteration of our arm: Chebyshev semi-iteration of the increment
# (--no-chebyshev: the reference's plain iteration); the CPU reference arm
# and the plain FP64 comparison always run the reference's iteration
CHEBYSHEV = 1
# the elastic warm start extrapolated to fifth order from the last six
# solutions (same fixed point and stopping test, fewer iterations when the
# fields move: 8.14 iterations per step over 100 steps at 246^3 against
# 11.1 with the linear form, fields against plain FP64 unchanged);
# --extrapolate-order 1..4: lower orders; --no-extrapolate: the reference's
# previous-solution start
EXTRAPOLATE = 5
# the 41-point stage of the 246-point transforms on the tensor cores
# (split-precision TF32); --fft-tensor-cores overrides
FFT_TENSOR_CORES = 0
# the generic engine's tile autotuner (--fft-autotune); off by default
FFT_AUTOTUNE = 0


def make_params(capi, n, precision, tol, shape=None, chebyshev=None):
    p = capi.load_params_file(PARAMS)
    p.Nx, p.Ny, p.Nz = shape if shape else (n, n, n)
    p.model_mode = capi.MODEL_GP_ZONE
    p.zero_mode_enabled = 1
    p.precision = capi.PREC_FP32 if precision == "fp32" else capi.PREC_FP64
    p.elastic_residual_tolerance = tol
    # with FP32 elastic fields the residual levels off near 8e-8 at 246^3, so
    # a 1e-8 tolerance runs to elastic_iter_max; the step continues there
    p.elastic_fail_on_nonconvergence = 0
    p.elastic_chebyshev = CHEBYSHEV if chebyshev is None else chebyshev
    p.elastic_warm_start_extrapolate = EXTRAPOLATE if chebyshev is None else 0
    p.fft_tensor_cores = FFT_TENSOR_CORES if chebyshev is None else 0
    p.fft_autotune = FFT_AUTOTUNE
    capi.finalize(p)
    return p


# population of the generated microstructure (set from the command line)
POPULATION = {"particles": None, "median_r": 6.0, "eta_sites": None}


def make_fields(capi, p, n, seed=2468):
    from cuda_sto_pf_gb300 import workloads
    shape = (p.Nx, p.Ny, p.Nz)
    frac = shape[0] * shape[1] * shape[2] / 246.0 ** 3
    count = POPULATION["particles"] or max(1, int(round(60 * frac)))
    sites = POPULATION["eta_sites"] or max(1, int(round(20 * frac)))
    w = workloads.ellipsoid_population(n, count=count, median_r=POPULATION["median_r"], eta_sites=sites,
                                       w=p.ic_phi_iface_w, seed=seed, shape=shape)
    phi, xB, eta = w["phi"], w["xB"], w["eta"]
    # raw-field rules of the reference loader (xB capped at its default
    # xB_max_safe = 0.07)
    st = capi.load().pfgb_prepare_raw_fields(ctypes.byref(p), 0.07, phi.ctypes.data, xB.ctypes.data,
                                             eta.ctypes.data, None, phi.size)
    assert st == 0
    return phi, xB, eta, w["n_particles"], w["n_eta"]


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(tag, shape):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)
    of kernel `tag` at `shape`, from the ncu summaries in profiles/ (lines
    `roofline-traffic: <tag> <Nx>x<Ny>x<Nz> <bytes>`); None if not captured."""
    key = "x".join(map(str, shape))
    pdir = os.path.join(REPO, "profiles")
    try:
        names = sorted(os.listdir(pdir))
    except OSError:
        return None
    for nm in names:
        if not nm.endswith((".md", ".txt")):
            continue
        with open(os.path.join(pdir, nm)) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 4 and parts[0] == "roofline-traffic:" and parts[1] == tag and parts[2] == key:
                    return {"bytes_per_launch": float(parts[3]), "source": f"profiles/{nm}"}
    return None


def cpu_oracle_rate(capi, n, precision, tol, threads=None, steps=1):
    """Oracle (FP64 CPU restatement) cell-steps/s on a bounded sample: one
    warm-up step (cold elastic start) + `steps` timed steps at n^3."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    from oracle_py import Oracle
    p = make_params(capi, n, precision, tol, chebyshev=0)
    phi, xB, eta, _, _ = make_fields(capi, p, n)
    threads = threads or os.cpu_count() or 1
    o = Oracle(p, threads=threads)
    o.load(phi, xB, eta)
    st = capi.StepStats()
    o.step(1, st)
    t0 = time.perf_counter()
    rc = o.step(steps, st)
    dt = time.perf_counter() - t0
    return {"value": n ** 3 * steps / dt, "unit": "cell-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} warm step(s) of the workload generator at {n}^3 (same parameters; "
                      f"one cold step untimed), FP64 oracle, {threads} OpenMP threads, rc={rc}",
            "seconds": dt}


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from cuda_sto_pf_gb300 import capi
    capi.load(build_if_missing=True)
    threads = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    from oracle_py import Oracle
    n = args.cpu_sample_n
    p = make_params(capi, n, args.precision, args.elastic_tol, chebyshev=0)
    phi, xB, eta, _, _ = make_fields(capi, p, n)
    o = Oracle(p, threads=threads)
    o.load(phi, xB, eta)
    st = capi.StepStats()
    for _ in range(args.warmup):
        o.step(1, st)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step(1, st)
    dt = time.perf_counter() - t0
    v = n ** 3 * args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cell-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded microstructure generator)",
            "config": {"workload": f"gp_zone dynamics, {n}^3 sample of the 246^3 workload", "grid": n,
                       "reference_cpu_path": "none in the reference (GPU-only code); the CPU oracle port "
                                             "restates its time step"},
            "cpu_baseline": {"value": v, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                             "sample": f"each step: one full dynamics step at {n}^3 (the 246^3 step "
                                       f"does not fit the time budget on the host cores)"},
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def short_run(capi, Solver, n, shape, fields, dev, stream, prec, tol, nsteps, warm, read=True, chebyshev=None):
    """nsteps steps from the initial fields; CUDA-event time per step over
    the last nsteps - warm; optionally the final fields and stress."""
    import torch
    p = make_params(capi, n, prec, tol, shape, chebyshev=chebyshev)
    s = Solver(p, device=dev)
    s.set_stream(stream.cuda_stream)
    s.load(*fields)
    iters = [s.step(1).elastic_iterations for _ in range(warm)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(nsteps - warm):
        iters.append(s.step(1).elastic_iterations)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / (nsteps - warm)
    f = s.fields() if read else None
    sig = s.elastic()["sigma"] if read else None
    s.close()
    return f, sig, ms, iters


def compare_plain_fp64(args, capi, Solver, n, shape, fields, dev, stream, nsteps=8, warm=3):
    """The chosen path (FP32 fields) and the plain FP64 form from the same
    initial fields on the same GPU: time per step of each over the last
    nsteps - warm steps, and the relative L2 field error of the chosen path
    against FP64 after nsteps steps."""
    res = {prec: short_run(capi, Solver, n, shape, fields, dev, stream, prec, args.elastic_tol, nsteps, warm,
                           chebyshev=None if prec == "fp32" else 0)
           for prec in ("fp32", "fp64")}
    f32, s32, ms32, it32 = res["fp32"]
    f64, s64, ms64, it64 = res["fp64"]
    N = shape[0] * shape[1] * shape[2]
    err = {k: rel_l2(f32[k], f64[k]) for k in ("phi", "xB", "eta")}
    err["sigma"] = rel_l2(s32, s64)
    return {"plain_fp64": {"value": N / (ms64 / 1e3), "unit": "cell-steps/s", "ms_per_step": ms64,
                           "elastic_iters_per_step": sum(it64[warm:]) / max(1, nsteps - warm)},
            "chosen_same_run": {"value": N / (ms32 / 1e3), "ms_per_step": ms32,
                                "elastic_iters_per_step": sum(it32[warm:]) / max(1, nsteps - warm)},
            "speedup_vs_plain_fp64": ms64 / ms32,
            "field_rel_l2_vs_fp64": err, "after_steps": nsteps,
            "what": f"the chosen path and the plain FP64 form with the reference's elastic iteration, from the "
                    f"same initial fields, {nsteps} steps; time over the last {nsteps - warm}; relative L2 error "
                    f"of phi, xB, eta and the 6 stress components"}


def run_horizon(args):
    """Field error of the chosen path (FP32 fields, Chebyshev increment
    iteration, extrapolated start) against the plain FP64 form (FP64
    fields, the reference's iteration) over a long horizon: both run the
    workload from the same initial fields side by side; the relative L2
    errors of phi, xB, eta and the six stress components are taken at
    several step counts."""
    import torch
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from cuda_sto_pf_gb300 import capi
    from cuda_sto_pf_gb300.solver import Solver
    capi.load(build_if_missing=True)
    torch.cuda.set_device(local)
    n = args.n
    shape = tuple(int(x) for x in args.shape.split(",")) if args.shape else (n, n, n)
    # the chosen arm: FP32 fields with the Chebyshev iteration and the
    # extrapolated start (default); fp64 = the same scheme in FP64 (isolates
    # the scheme); fp64-plain = the plain FP64 form at --elastic-tol (with
    # --horizon-plain-tol: the trajectory's sensitivity to the elastic tolerance)
    chosen = args.horizon_chosen
    if chosen == "fp64-plain":
        p32 = make_params(capi, n, "fp64", args.elastic_tol, shape, chebyshev=0)
    else:
        p32 = make_params(capi, n, "fp32" if chosen == "fp32" else "fp64", args.elastic_tol, shape)
    plain_tol = args.horizon_plain_tol or args.elastic_tol
    p64 = make_params(capi, n, "fp64", plain_tol, shape, chebyshev=0)
    phi, xB, eta, npart, neta = make_fields(capi, p32, n)
    marks = sorted(set(int(x) for x in args.horizon_marks.split(",")))
    stream = torch.cuda.current_stream(local)
    out = []
    it32, it64, conv32, ms32, ms64 = [], [], 0, 0.0, 0.0
    unconv = []   # steps (1-based) of the chosen arm that ended at the iteration cap
    with Solver(p32, device=local) as s32, Solver(p64, device=local) as s64:
        for s in (s32, s64):
            s.set_stream(stream.cuda_stream)
            s.load(phi, xB, eta)
        done = 0
        for m in marks:
            for _ in range(m - done):
                for s, its, tag in ((s32, it32, 32), (s64, it64, 64)):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    st = s.step(1)
                    e1.record(stream)
                    e1.synchronize()
                    its.append(st.elastic_iterations)
                    if tag == 32:
                        ms32 += e0.elapsed_time(e1)
                        conv32 += st.elastic_converged
                        if not st.elastic_converged:
                            unconv.append(len(it32))
                    else:
                        ms64 += e0.elapsed_time(e1)
            done = m
            f32, f64 = s32.fields(), s64.fields()
            err = {k: rel_l2(f32[k], f64[k]) for k in ("phi", "xB", "eta")}
            err["sigma"] = rel_l2(s32.elastic()["sigma"], s64.elastic()["sigma"])
            m32, m64 = s32.diagnostics().mass_xBtot, s64.diagnostics().mass_xBtot
            err["mass_rel_fp32_vs_fp64"] = abs(m32 - m64) / m64
            out.append({"after_steps": m, "field_rel_l2_vs_fp64": err})
            print(json.dumps({"after_steps": m, **err}), file=sys.stderr, flush=True)
    line = {"metric": f"field rel. L2 of the chosen path ({chosen}) vs the plain FP64 form over a long horizon",
            "value": out[-1]["field_rel_l2_vs_fp64"]["xB"], "unit": "relative L2 (xB)", "n_gpus": 1,
            "steps": marks[-1], "warmup": 0, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if chosen == "fp32" else "f64",
            "data": "synthetic (seeded microstructure generator, reference raw-field rules)",
            "config": {"workload": f"{'x'.join(map(str, shape))} gp_zone dynamics, {npart} ellipsoids + "
                                   f"{neta} eta sites, heterogeneous elasticity, zero mode",
                       "chosen": chosen, "elastic_tol": args.elastic_tol, "plain_fp64_elastic_tol": plain_tol,
                       "dt": p32.dt},
            "horizon": out,
            "chosen": {"ms_per_step": ms32 / marks[-1], "elastic_iters_per_step": sum(it32) / len(it32),
                       "elastic_converged_steps": conv32, "nonconverged_steps": unconv,
                       "elastic_iters": it32},
            "plain_fp64": {"ms_per_step": ms64 / marks[-1], "elastic_iters_per_step": sum(it64) / len(it64)}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    global FFT_TENSOR_CORES
    if args.fft_tensor_cores is not None:
        FFT_TENSOR_CORES = args.fft_tensor_cores
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
    dev = local
    torch.cuda.set_device(dev)
    from cuda_sto_pf_gb300 import capi
    from cuda_sto_pf_gb300.solver import Solver
    capi.load(build_if_missing=True)
    n = args.n
    shape = tuple(int(x) for x in args.shape.split(",")) if args.shape else (n, n, n)
    N = shape[0] * shape[1] * shape[2]
    p = make_params(capi, n, args.precision, args.elastic_tol, shape)
    phi, xB, eta, npart, neta = make_fields(capi, p, n)
    stream = torch.cuda.current_stream(dev)
    s = Solver(p, device=dev)
    s.set_stream(stream.cuda_stream)
    s.load(phi, xB, eta)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize(dev)

    stats = capi.StepStats()
    iters = []
    for _ in range(max(args.warmup, 3)):
        stats = s.step(1)
    # ---- device-resident timed region --------------------------------------
    clocks = Clocks(dev)
    barrier()
    clocks.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.profile_enable(False)   # resets the launch counter; no per-launch events in the timed region
    ev0.record(stream)
    w0 = time.perf_counter()
    conv, resid = [], []
    for _ in range(args.steps):
        st = s.step(1)
        iters.append(st.elastic_iterations)
        conv.append(st.elastic_converged)
        resid.append(st.elastic_relative_residual)
    ev1.record(stream)
    barrier()
    wall = time.perf_counter() - w0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    launches = s.launches()
    dev_bytes = int(capi.load().pfgb_device_bytes(s.ctx))
    # per-kernel CUDA-event timing on a separate pass (events bracket every launch)
    s.profile_enable(True)
    for _ in range(min(args.steps, 5)):
        s.step(1)
    prof = s.profile_read()
    prof_steps = min(args.steps, 5)
    s.profile_enable(False)
    t = torch.tensor([ms], device=f"cuda:{dev}")
    if ws > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = ws * N * args.steps / (ms_max / 1e3)

    # ---- e2e through the C ABI with pinned host buffers --------------------
    e2e = None
    if not args.no_e2e:
        pin = {k: torch.empty(N, dtype=torch.float64).pin_memory() for k in ("phi", "xB", "Y", "eta", "dYdt")}
        s.read_into(pin["phi"].data_ptr(), pin["xB"].data_ptr(), pin["Y"].data_ptr(), pin["eta"].data_ptr(),
                    pin["dYdt"].data_ptr())
        h2d = 4 * N * 8
        d2h = 5 * N * 8
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            s.set_fields(pin["phi"].data_ptr(), pin["xB"].data_ptr(), pin["eta"].data_ptr(), pin["dYdt"].data_ptr())
            s.step_nostats(1)
            s.read_into(pin["phi"].data_ptr(), pin["xB"].data_ptr(), pin["Y"].data_ptr(), pin["eta"].data_ptr(),
                        pin["dYdt"].data_ptr())
        e1.record(stream)
        barrier()
        ems = e0.elapsed_time(e1)
        te = torch.tensor([ems], device=f"cuda:{dev}")
        if ws > 1:
            import torch.distributed as dist
            dist.all_reduce(te, op=dist.ReduceOp.MAX)
        e2e = {"value": ws * N * args.steps / (float(te.item()) / 1e3), "unit": "cell-steps/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "what": "per step: pfgb_set_fields (4 float64 fields from pinned host) + pfgb_step + "
                       "pfgb_read_fields (5 float64 fields to pinned host)"}

    # ---- roofline of the dominant kernel ------------------------------------
    peak, peak_kind = measured_peak()
    prof.sort(key=lambda r: -r["ms"])
    total_ms = sum(r["ms"] for r in prof) or 1.0
    top = prof[0] if prof else None
    roof = None
    if top:
        achieved = top["bytes"] / (top["ms"] / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": top["kernel"], "achieved": achieved, "peak": peak,
                "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                "traffic": None, "traffic_source": None,
                "share": top["ms"] / total_ms,
                "algorithmic_bytes_per_launch": top["bytes"] / max(1, top["launches"]),
                "avg_launch_ms": top["ms"] / max(1, top["launches"])}
        tr = ncu_traffic(top["kernel"], shape)
        if tr:
            roof["traffic"] = tr["bytes_per_launch"]
            roof["traffic_source"] = tr["source"]
    if args.profile_json and rank == 0:
        with open(args.profile_json, "w") as f:
            json.dump({"kernels": prof, "total_ms": total_ms, "launches": launches, "steps": args.steps,
                       "profiled_steps": prof_steps, "iters": iters}, f, indent=1)

    s.close()
    plain = None
    ref_tol = None
    if rank == 0 and not args.no_plain_fp64:
        plain = compare_plain_fp64(args, capi, Solver, n, shape, (phi, xB, eta), dev, stream)
        # the same step at the reference's default elastic tolerance (1e-6)
        _, _, ms6, it6 = short_run(capi, Solver, n, shape, (phi, xB, eta), dev, stream, args.precision, 1e-6,
                                   8, 3, read=False)
        ref_tol = {"elastic_tol": 1e-6, "value": N / (ms6 / 1e3), "unit": "cell-steps/s", "ms_per_step": ms6,
                   "elastic_iters_per_step": sum(it6[3:]) / 5.0}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_oracle_rate(capi, args.cpu_sample_n, args.precision, args.elastic_tol)
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "cell-steps/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {e}"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": ws, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32" if args.precision == "fp32" else "f64",
                "data": "synthetic (seeded microstructure generator, reference raw-field rules)",
                "config": {"workload": f"{'x'.join(map(str, shape))} gp_zone dynamics, {npart} ellipsoids + {neta} eta sites, "
                                       f"heterogeneous elasticity, zero mode",
                           "grid": n, "fields": args.precision, "elastic": "fp32",
                           "elastic_tol": args.elastic_tol, "dt": p.dt,
                           "elastic_iteration": "chebyshev semi-iteration of the increment" if CHEBYSHEV
                           else "plain (the reference's)",
                           "elastic_warm_start": {0: "previous solution (the reference's)",
                                                  1: "extrapolated linearly from the last two solutions",
                                                  2: "extrapolated quadratically from the last three solutions",
                                                  3: "extrapolated cubically from the last four solutions",
                                                  4: "extrapolated to fourth order from the last five solutions",
                                                  5: "extrapolated to fifth order from the last six solutions"
                                                  }[EXTRAPOLATE],
                           "fft_autotune": FFT_AUTOTUNE,
                           "dft41_stage": "tensor cores (tcgen05, split-precision TF32)" if FFT_TENSOR_CORES
                           else "FP32 multiply-adds",
                           "l2": "inputs larger than L2 (working set > 1 GB at 246^3)",
                           "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
                "elastic_iters_per_step": sum(iters) / max(1, len(iters)),
                # every timed step's elastic solve against the tolerance (the
                # step continues at the cap, so this is the check)
                "elastic_converged_steps": int(sum(conv)), "elastic_timed_steps": len(conv),
                "elastic_max_final_residual": max(resid) if resid else None,
                "elastic_max_iters": max(iters) if iters else None,
                # summed per-launch kernel time over the step time: the rest is
                # host round trips (residual reads, zero-mode scalars) and gaps
                "kernel_busy_fraction": (total_ms / max(1, prof_steps)) / (ms_max / args.steps),
                "wall_ms_per_step": 1e3 * wall / args.steps,
                "device_bytes": dev_bytes,
                "gpu_launches": launches,
                "tiles": capi.tile_report().splitlines() if FFT_AUTOTUNE else [],
                "clocks": clk, "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "vs_plain_fp64": plain,
                "at_reference_default_tol": ref_tol}
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_sweep(args):
    """Batched minimize sweep: 48 cases of 64^3-160^3 (sphere / oblate
    spheroid seeds, eigenstrain rotated by 8 seeded rotations), 500 minimize
    iterations each at dt 0.05, V0 0.1, full model, FP32 fields, through
    pfgb_batch_minimize (host fields in and out)."""
    import torch
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from cuda_sto_pf_gb300 import capi, workloads
    lib = capi.load(build_if_missing=True)
    specs = workloads.sweep_cases(count=args.sweep_cases)
    arr = (capi.Case * len(specs))()
    keep = []
    for i, c in enumerate(specs):
        f = workloads.spheroid_fields(c)
        p = capi.load_params_file(PARAMS)
        p.Nx = p.Ny = p.Nz = c["n"]
        p.mode = capi.MODE_MINIMIZE
        p.minimize_full_model = 1
        p.minimize_dt = 0.05
        p.minimize_V0 = 0.1
        p.precision = capi.PREC_FP32
        p.fft_autotune = args.sweep_autotune
        for k in range(6):
            p.eps00[k] = c["eps00"][k]
        capi.finalize(p)
        lib.pfgb_prepare_raw_fields(ctypes.byref(p), 0.07, f["phi"].ctypes.data, f["xB"].ctypes.data, None, None,
                                    f["phi"].size)
        out = np.empty_like(f["phi"])
        keep.append((f, out))
        arr[i].params = p
        arr[i].phi = f["phi"].ctypes.data
        arr[i].xB = f["xB"].ctypes.data
        arr[i].phi_out = out.ctypes.data
        arr[i].max_iter = args.sweep_iters
        arr[i].stop_on_convergence = 0   # fixed iteration count, as the config times it
    cell_its = sum(c["n"] ** 3 for c in specs) * args.sweep_iters
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc = lib.pfgb_batch_minimize(arr, len(specs), local, args.sweep_concurrency)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ok = sum(1 for i in range(len(specs)) if arr[i].status == 0)
    v = cell_its / wall
    line = {"metric": "cell-iterations/s (batched minimize sweep)", "value": v, "unit": "cell-iterations/s",
            "n_gpus": 1, "steps": args.sweep_iters, "warmup": 0, "ms_per_step": 1e3 * wall / args.sweep_iters,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded sweep cases)",
            "config": {"workload": f"{len(specs)} minimize cases, grids 64^3-160^3, sphere/oblate seeds, "
                                   f"8 eigenstrain rotations, {args.sweep_iters} iterations, dt 0.05, V0 0.1, "
                                   f"full model", "concurrency": args.sweep_concurrency,
                       "fft_autotune": args.sweep_autotune,
                       "l2": "per-case working sets 0.2-1 GB, above L2"},
            "e2e": {"value": v, "unit": "cell-iterations/s",
                    "h2d_bytes_per_step": 2 * 8 * sum(c["n"] ** 3 for c in specs) / args.sweep_iters,
                    "d2h_bytes_per_step": 8 * sum(c["n"] ** 3 for c in specs) / args.sweep_iters,
                    "what": "host raw fields in, final phi out, through pfgb_batch_minimize; the whole sweep is "
                            "one call, so this equals value"},
            "cases_ok": ok, "status": rc,
            "case_seconds": [round(arr[i].seconds, 3) for i in range(len(specs))],
            "tiles": capi.tile_report().splitlines() if args.sweep_autotune else [],
            "roofline": None, "cpu_baseline": None}
    print(json.dumps(line), flush=True)


def _fno_micro(args):
    """One seeded C1-like microstructure (5-30 ellipsoids, GP-zone eta seeds)
    as float32 arrays; runs in a worker process."""
    n, seed, w = args
    from cuda_sto_pf_gb300 import workloads
    rng = np.random.default_rng(seed)
    count = int(rng.integers(5, 31))
    m = workloads.ellipsoid_population(n, count=count, eta_sites=max(1, count // 3), w=w, seed=seed)
    return tuple(m[k].astype(np.float32) for k in ("phi", "xB", "eta"))


def _cube_symmetry(fields, k):
    """The k-th of the 48 symmetries of the cube (axis permutation + flips)."""
    import itertools
    perm = list(itertools.permutations((0, 1, 2)))[k % 6]
    flips = [a for a in range(3) if (k // 6) >> a & 1]
    return tuple(np.ascontiguousarray(np.flip(np.transpose(f, perm), axis=flips) if flips else np.transpose(f, perm))
                 for f in fields)


def run_fno(args):
    """Learned elastic start at 128^3: a 4-layer FNO (width 32, 12 modes,
    bfloat16 weights) fitted on pairs from the solver's own cold elastic
    solves of C1-like microstructures (5-30 particles, cube-symmetry copies
    of the generated ones), then dynamics steps of held-out microstructures
    started cold, from the previous step (the reference's warm start) and
    from the model, all to the same residual tolerance."""
    import multiprocessing as mp
    ws, rank, local = dist_env()
    if rank != 0:
        return
    n = args.fno_n
    # microstructures first, in spawned workers, before any GPU call
    nbase = args.fno_base
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        base = pool.map(_fno_micro, [(n, 5000 + i, 2.5) for i in range(nbase + 2)])
    import torch
    from cuda_sto_pf_gb300 import capi, fno
    from cuda_sto_pf_gb300.solver import Solver
    lib = capi.load(build_if_missing=True)
    torch.cuda.set_device(local)
    p = make_params(capi, n, "fp32", args.elastic_tol)
    N = n ** 3

    def prepared(fields):
        phi, xB, eta = (np.ascontiguousarray(f, dtype=np.float64) for f in fields)
        assert lib.pfgb_prepare_raw_fields(ctypes.byref(p), 0.07, phi.ctypes.data, xB.ctypes.data,
                                           eta.ctypes.data, None, phi.size) == 0
        return phi, xB, eta

    P = args.fno_pairs
    inputs = torch.empty((P, 8, N), device="cuda")
    targets = torch.empty((P, 3, N), device="cuda")
    t0 = time.perf_counter()
    cold_its = []
    with Solver(p, device=local) as s:
        for i in range(P):
            s.load(*prepared(_cube_symmetry(base[i % nbase], i // nbase)))
            st = s.training_pair(inputs[i], targets[i])
            cold_its.append(st.elastic_iterations)
        s.sync()
    t_pairs = time.perf_counter() - t0
    hold = P // 16
    in_scale, out_scale = fno.channel_scales(inputs[hold:], targets[hold:])
    model = fno.WarmStartModel((n, n, n), modes=12, layers=4, in_scale=in_scale, out_scale=out_scale, device=local)
    t0 = time.perf_counter()
    losses = fno.train(model, inputs[hold:], targets[hold:], steps=args.fno_train_steps, lr=1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    # held-out relative error of the prediction
    pred = torch.empty((3, N), device="cuda")
    errs = []
    for i in range(hold):
        model.forward(inputs[i], pred)
        errs.append(float((pred - targets[i]).norm() / targets[i].norm()))
    fwd_ms = []
    for _ in range(5):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        model.forward(inputs[0], pred)
        b.record()
        torch.cuda.synchronize()
        fwd_ms.append(a.elapsed_time(b))
    del inputs, targets
    torch.cuda.empty_cache()
    # dynamics from the two held-out generated microstructures
    modes = {"cold": 3, "previous_step": 0, "model_every_step": 2, "model_cold_start_then_previous": 1}
    res = {}
    for name, src in modes.items():
        pm = make_params(capi, n, "fp32", args.elastic_tol)
        pm.elastic_warm_start_source = src
        its, ms, first, err = [], [], [], None
        for k in range(2):
            with Solver(pm, device=local) as s:
                s.set_warm_start_model(model)
                s.load(*prepared(base[nbase + k]))
                try:
                    for j in range(args.fno_eval_steps):
                        torch.cuda.synchronize()
                        t1 = time.perf_counter()
                        st = s.step(1)
                        torch.cuda.synchronize()
                        ms.append(1e3 * (time.perf_counter() - t1))
                        its.append(st.elastic_iterations)
                        if j == 0:
                            first.append(st.elastic_iterations)
                except capi.PfgbError as e:
                    err = str(e)
                s.set_warm_start_model(None)
        res[name] = {"iterations_per_step": float(np.mean(its)) if its else None,
                     "ms_per_step": float(np.mean(ms)) if ms else None,
                     "first_step_iterations": first, "steps": len(its), "error": err}
    model.close()
    line = {"metric": "elastic iterations per step (learned start)",
            "value": res["model_every_step"]["iterations_per_step"], "unit": "iterations/step",
            "higher_is_better": False, "n_gpus": 1, "steps": args.fno_eval_steps, "dtype": "f32",
            "data": "synthetic (seeded C1-like microstructures, cube-symmetry copies)",
            "config": {"workload": f"{n}^3 gp_zone dynamics, heterogeneous elasticity, zero mode, elastic tol "
                                   f"{args.elastic_tol:g}; FNO width 32, 12 modes, 4 layers, bf16 weights",
                       "pairs": P, "held_out_pairs": hold, "distinct_microstructures": nbase,
                       "train_steps": args.fno_train_steps},
            "starts": res,
            "model": {"held_out_rel_l2": float(np.mean(errs)), "forward_ms": float(np.median(fwd_ms)),
                      "train_loss_first_100": float(np.mean(losses[:100])),
                      "train_loss_last_100": float(np.mean(losses[-100:])),
                      "pair_cold_iterations_mean": float(np.mean(cold_its)),
                      "seconds_pairs": t_pairs, "seconds_train": t_train}}
    print(json.dumps(line), flush=True)


def run_fno_step(args):
    """Cost of the learned start's kernels at --fno-n: one forward (the
    solver's use) and one training step (forward, backward, Adam) on seeded
    random inputs, CUDA-event timed after --warmup repeats."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    import torch
    from cuda_sto_pf_gb300 import capi, fno
    capi.load(build_if_missing=True)
    torch.cuda.set_device(local)
    n = args.fno_n
    N = n ** 3
    g = torch.Generator(device="cuda").manual_seed(1)
    x = torch.randn((8, N), device="cuda", generator=g)
    t = torch.randn((3, N), device="cuda", generator=g)
    y = torch.empty((3, N), device="cuda")
    model = fno.WarmStartModel((n, n, n), modes=12, layers=4, device=local)

    def timed(fn, reps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    fwd = timed(lambda: model.forward(x, y), args.steps)
    trn = timed(lambda: (model.loss_grad(x, t, want_loss=False), model.adam_step(1e-5)), max(1, args.steps // 2))
    model.close()
    print(json.dumps({"metric": "learned-start model cost", "grid": n, "forward_ms": fwd, "train_step_ms": trn,
                      "steps": args.steps, "warmup": args.warmup}), flush=True)


def main():
    global CHEBYSHEV, EXTRAPOLATE, FFT_AUTOTUNE
    args = parse()
    POPULATION.update(particles=args.particles, median_r=args.median_radius, eta_sites=args.eta_sites)
    CHEBYSHEV = 0 if args.no_chebyshev else 1
    FFT_AUTOTUNE = args.fft_autotune
    if args.no_extrapolate:
        EXTRAPOLATE = 0
    elif args.extrapolate_order:
        EXTRAPOLATE = args.extrapolate_order
    if args.workload == "horizon":
        run_horizon(args)
        return
    if args.workload == "sweep":
        run_sweep(args)
        return
    if args.workload == "fno":
        run_fno(args)
        return
    if args.workload == "fno-step":
        run_fno_step(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
