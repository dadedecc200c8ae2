"""Build recipe for the CPU oracle (test infrastructure, not the product).

    python oracle/build_oracle.py          # -> oracle/_build/libpforacle.so
    python oracle/build_oracle.py --ref    # also oracle/_ref/libpfref.so, libpfckpt.so

The oracle is plain C99 + OpenMP.  FP contraction is disabled so x86 and
aarch64 builds give the same roundings.  ``--ref`` compiles the reference's
own thermo_utils.h / phase_functions.h (read in place under the reference
tree; nothing is copied) into oracle/_ref/ for pinning the restatement,
and the reference's pf_zero_mode_checkpoint.cpp (also read in place) with
the shim ckpt_ref_shim.cpp into oracle/_ref/libpfckpt.so for pinning the
checkpoint files.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "libpforacle.so")
REF_LIB = os.path.join(REF_OUT, "libpfref.so")
CKPT_LIB = os.path.join(REF_OUT, "libpfckpt.so")
REFERENCE_TREE = "/root/reference"

CFLAGS = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
          "-fno-fast-math", "-Wall", "-Wno-unused-function"]


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "pf_oracle.c"), os.path.join(HERE, "pf_fft.c")]
    deps = srcs + [os.path.join(HERE, "pf_oracle.h"),
                   os.path.join(HERE, "..", "include", "pfgb.h")]
    if force or _stale(LIB, deps):
        tmp = LIB + ".tmp"
        subprocess.run(["gcc", *CFLAGS, "-o", tmp, *srcs, "-lm"], check=True)
        os.replace(tmp, LIB)
    return LIB


def build_ref(force: bool = False) -> str | None:
    """Compile the reference's host-callable thermo/phase headers.

    Only possible where the reference tree is present; returns None
    otherwise.  The shim (ref_pin.c) defines away the CUDA qualifiers and
    includes the headers from the reference tree by absolute path.
    """
    if not os.path.isdir(REFERENCE_TREE):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    shim = os.path.join(HERE, "ref_pin.c")
    hdrs = [os.path.join(REFERENCE_TREE, "thermo_utils.h"),
            os.path.join(REFERENCE_TREE, "phase_functions.h")]
    if force or _stale(REF_LIB, [shim]):
        tmp = REF_LIB + ".tmp"
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                        "-I", REFERENCE_TREE, "-o", tmp, shim, "-lm"], check=True)
        os.replace(tmp, REF_LIB)
    del hdrs
    return REF_LIB


def build_ref_checkpoint(force: bool = False) -> str | None:
    """Compile the reference's checkpoint writer/reader with the test shim.

    Only where the reference tree is present; returns None otherwise."""
    src = os.path.join(REFERENCE_TREE, "pf_zero_mode_checkpoint.cpp")
    if not os.path.exists(src):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    shim = os.path.join(HERE, "ckpt_ref_shim.cpp")
    if force or _stale(CKPT_LIB, [shim, os.path.join(HERE, "..", "include", "pfgb.h")]):
        tmp = CKPT_LIB + ".tmp"
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", REFERENCE_TREE, "-o", tmp, shim, src],
                       check=True)
        os.replace(tmp, CKPT_LIB)
    return CKPT_LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    if "--ref" in sys.argv:
        print(build_ref(force="--force" in sys.argv))
        print(build_ref_checkpoint(force="--force" in sys.argv))
