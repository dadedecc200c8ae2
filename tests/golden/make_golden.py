"""Regenerate the committed golden fixtures in tests/golden/.

Run in a container that has the reference tree (it is read, never copied):

    python oracle/build_oracle.py --ref
    python tests/golden/make_golden.py

Outputs
  c1.params, c2.params      -- main_cuda `key=value` parameter files produced by
                               the reference's own converter
                               (Unit_Psedobinary.py generate_payload +
                               write_main_cuda_override_file) for the workload
                               physical inputs below.
  thermo_golden.json        -- pointwise thermodynamics / phase functions
                               evaluated by the reference headers compiled on
                               the host (oracle/_ref/libpfref.so).

Physical basis of the parameter files: the reference's
physical_inputs.example.json with dx = 1 nm (pf_dx = phys_dx_ref = 1e-9 m),
lambda_sm = 5 nm, the cubic stiffness tensors of each workload and the
eigenstrain diag(0.046, -0.022, -0.017).
"""
from __future__ import annotations

import ctypes
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.abspath(os.path.join(HERE, "..", ".."))
REFERENCE_TREE = os.environ.get("PFGB_REFERENCE_TREE") or os.path.normpath(
    os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "..", "reference"))


def cubic(c11: float, c12: float, c44: float) -> list[list[float]]:
    return [[c11, c12, c12, 0, 0, 0], [c12, c11, c12, 0, 0, 0], [c12, c12, c11, 0, 0, 0],
            [0, 0, 0, c44, 0, 0], [0, 0, 0, 0, c44, 0], [0, 0, 0, 0, 0, c44]]


def physical_inputs(c_matrix, c_precip) -> dict:
    with open(os.path.join(REFERENCE_TREE, "physical_inputs.example.json")) as f:
        base = json.load(f)
    base = {k: v for k, v in base.items() if not k.startswith("_")}
    base.update({
        "dx": 1e-9, "pf_dx": 1e-9, "phys_dx_ref": 1e-9, "lambda_sm": 5e-9,
        "eigenstrain_principal": [0.046, -0.022, -0.017],
        "eigenstrain_rotation_matrix": [[1, 0, 0], [0, 1, 0], [0, 0, 1]],
        "C_tensor_PbTe_GPa": c_matrix, "C_tensor_Ag2Te_GPa": c_precip,
    })
    base.pop("eigenstrain_tensor", None)
    return base


def make_params() -> None:
    sys.path.insert(0, REFERENCE_TREE)
    import Unit_Psedobinary as up  # the reference converter, imported in place

    pbte = cubic(108.0, 7.7, 13.0)
    cases = {
        "c1.params": physical_inputs(pbte, pbte),                       # homogeneous
        "c2.params": physical_inputs(pbte, cubic(60.0, 25.0, 15.0)),    # S_p != 0
    }
    for name, phys in cases.items():
        known = set(up.PhysicalInputs.__dataclass_fields__.keys())
        phys = {k: v for k, v in phys.items() if k in known}
        inputs = up.PhysicalInputs(**phys)
        payload = up.generate_payload(inputs)
        up.write_main_cuda_override_file(os.path.join(HERE, name),
                                         payload["main_cuda_overrides"])
        print("wrote", name)


def make_thermo() -> None:
    lib = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libpfref.so"))
    d = ctypes.c_double
    for n, k in [("ref_h", 1), ("ref_hp", 1), ("ref_gp", 1), ("ref_xB_eq", 1),
                 ("ref_mu_A", 3), ("ref_mu_B", 3), ("ref_gamma", 7), ("ref_sigmoid", 3),
                 ("ref_logit", 3)]:
        f = getattr(lib, n)
        f.restype = d
        f.argtypes = [d] * k
    lib.ref_set_convex.argtypes = [ctypes.c_int]
    phis = [-0.1, 0.0, 1e-3, 0.1, 0.25, 0.5, 0.75, 0.9, 0.999, 1.0, 1.05]
    xs = [1e-14, 1e-9, 1e-4, 0.003, 0.0155, 0.03, 0.0799, 0.08, 0.0801, 0.0899, 0.09,
          0.0901, 0.12, 0.2, 0.33, 0.5, 0.9, 0.999999]
    Ts = [573.15, 653.15, 723.15, 1300.0]
    scales = [1.0, 5000.0, 17352.8741]
    out: dict = {"phase": [], "mu": [], "gamma": [], "xB_eq": [], "sigmoid": [], "logit": []}
    for p in phis:
        out["phase"].append([p, lib.ref_h(p), lib.ref_hp(p), lib.ref_gp(p)])
    for T in Ts:
        out["xB_eq"].append([T, lib.ref_xB_eq(T)])
    vm0, dvm, vmc = 1.0, -0.0412, 1.32
    for convex in (0, 1):
        lib.ref_set_convex(convex)
        for T in Ts:
            for s in scales:
                for x in xs:
                    out["mu"].append([convex, x, T, s, lib.ref_mu_A(x, T, s), lib.ref_mu_B(x, T, s)])
                    for h in (0.0, 0.37, 1.0):
                        out["gamma"].append([convex, x, h, vm0, dvm, vmc, T, s,
                                             lib.ref_gamma(x, h, vm0, dvm, vmc, T, s)])
    lib.ref_set_convex(0)
    for Y in [-40.0, -20.0, -19.9, -3.5, -1e-3, 0.0, 2.0, 19.0, 25.0]:
        for eps in (1e-8, 1e-12):
            out["sigmoid"].append([Y, 20.0, eps, lib.ref_sigmoid(Y, 20.0, eps)])
    for x in [0.0, 1e-12, 1e-8, 0.03, 0.33, 0.5, 0.99999999, 1.0]:
        out["logit"].append([x, 1e-8, 20.0, lib.ref_logit(x, 1e-8, 20.0)])
    with open(os.path.join(HERE, "thermo_golden.json"), "w") as f:
        json.dump(out, f, indent=0)
    print("wrote thermo_golden.json")


if __name__ == "__main__":
    make_params()
    make_thermo()
