"""Build recipe for the CPU oracle (test infrastructure, not the product).

    python oracle/build_oracle.py            # -> oracle/_build/libpforacle.so
    python oracle/build_oracle.py --ref      # also oracle/_ref/libpfref.so, libpfckpt.so, librefk.so
    python oracle/build_oracle.py --ref-main # stage the reference main_cuda sources and build it

The reference tree is $PFGB_REFERENCE_TREE, or else the checkout named
``reference`` beside this repository.

The oracle is plain C99 + OpenMP.  FP contraction is disabled so x86 and
aarch64 builds give the same roundings.  ``--ref`` compiles the reference's
own thermo_utils.h / phase_functions.h (read in place under the reference
tree; nothing is copied) into oracle/_ref/ for pinning the restatement,
and the reference's pf_zero_mode_checkpoint.cpp (also read in place) with
the shim ckpt_ref_shim.cpp into oracle/_ref/libpfckpt.so for pinning the
checkpoint files, and the kernel section of the reference's cuda_kernels.cu
(read in place, written to oracle/_ref/) with the shim ref_kernels.cpp into
oracle/_ref/librefk.so for pinning the oracle's per-cell physics.
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
KERN_LIB = os.path.join(REF_OUT, "librefk.so")
KERN_SECTION = os.path.join(REF_OUT, "ref_kernels_section.inc")
CUDA_INCLUDE = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
REFERENCE_TREE = os.environ.get("PFGB_REFERENCE_TREE") or os.path.normpath(
    os.path.join(HERE, "..", "..", "reference"))
# The reference's own GPU program, rebuilt for sm_103a as the whole-step
# oracle.  Its sources are staged (copied unchanged, git-ignored) into
# oracle/_ref/main_src/ where the reference tree is present, so that a
# machine without the tree (the GPU host) can still build it; the binary is
# named for the host architecture because it is rebuilt on each machine.
REF_MAIN_SOURCES = ["main_cuda.cu", "cuda_kernels.cu", "cuda_common.cu", "pf_zero_mode_checkpoint.cpp"]
REF_MAIN_HEADERS = ["cuda_common.h", "cuda_kernels.h", "pf_params.h", "phase_functions.h", "thermo_utils.h",
                    "io_vtk_cuda.h", "pf_zero_mode_checkpoint.h"]
REF_MAIN_SRC = os.path.join(REF_OUT, "main_src")
REF_MAIN_BIN = os.path.join(REF_OUT, "main_cuda_ref." + os.uname().machine)
NVCC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")

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


def _kernel_section(path: str) -> str:
    """The kernel section of the reference's cuda_kernels.cu: everything
    after its #include lines up to the first top-level definition that
    contains a kernel launch (the host launch wrappers)."""
    import re
    lines = open(path).read().split("\n")
    last_inc = max(i for i, l in enumerate(lines[:60]) if l.startswith("#include"))
    first_launch = next(i for i, l in enumerate(lines) if "<<<" in l)
    depth, starts = 0, []
    for i, l in enumerate(lines[:first_launch]):
        if depth == 0 and re.match(r"^[A-Za-z_]", l) and not l.startswith("#"):
            starts.append(i)
        depth += l.count("{") - l.count("}")
    out = lines[last_inc + 1:starts[-1]]
    # kernels defined among the launch wrappers, taken whole by name
    for name in ("compute_displacement_from_hij_green_kernel", "compute_strain_with_perturbation_kernel"):
        i0 = next(i for i, l in enumerate(lines) if l.startswith("__global__ void " + name + "("))
        depth, seen, i = 0, False, i0
        while True:
            depth += lines[i].count("{") - lines[i].count("}")
            seen = seen or "{" in lines[i]
            i += 1
            if seen and depth == 0:
                break
        out += lines[i0:i]
    return "\n".join(out) + "\n"


def build_ref_kernels(force: bool = False) -> str | None:
    """Compile the reference's per-cell kernels for the host (ref_kernels.cpp).

    The kernel section is read from cuda_kernels.cu where it lies and written
    to oracle/_ref/ (a build output, git-ignored); only where the reference
    tree and the CUDA headers are present; returns None otherwise."""
    src = os.path.join(REFERENCE_TREE, "cuda_kernels.cu")
    if not os.path.exists(src) or not os.path.isdir(CUDA_INCLUDE):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    shim = os.path.join(HERE, "ref_kernels.cpp")
    if force or _stale(KERN_LIB, [shim, src]):
        with open(KERN_SECTION, "w") as f:
            f.write(_kernel_section(src))
        tmp = KERN_LIB + ".tmp"
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w",
                        "-I", REFERENCE_TREE, "-I", REF_OUT, "-I", CUDA_INCLUDE, "-o", tmp, shim], check=True)
        os.replace(tmp, KERN_LIB)
    return KERN_LIB


def stage_ref_main() -> str | None:
    """Copy the reference main_cuda's source files, unchanged, into
    oracle/_ref/main_src/ (git-ignored).  Only where the reference tree is
    present; returns the staging directory, or None."""
    import shutil
    if not all(os.path.exists(os.path.join(REFERENCE_TREE, f)) for f in REF_MAIN_SOURCES + REF_MAIN_HEADERS):
        return None
    os.makedirs(REF_MAIN_SRC, exist_ok=True)
    for f in REF_MAIN_SOURCES + REF_MAIN_HEADERS:
        src, dst = os.path.join(REFERENCE_TREE, f), os.path.join(REF_MAIN_SRC, f)
        if _stale(dst, [src]):
            shutil.copyfile(src, dst + ".tmp")
            os.replace(dst + ".tmp", dst)
    return REF_MAIN_SRC


def build_ref_main(force: bool = False) -> str | None:
    """Build the reference main_cuda for sm_103a from the staged sources:
    nvcc on its four translation units with the flags of its Makefile
    (-O3 -std=c++14 --expt-relaxed-constexpr) and CUDA_ARCH=sm_103a, linked
    with cuFFT.  Returns the binary, or None when no staged sources exist
    (no reference tree here and none staged before)."""
    stage_ref_main()
    srcs = [os.path.join(REF_MAIN_SRC, f) for f in REF_MAIN_SOURCES]
    if not all(os.path.exists(f) for f in srcs) or not os.path.exists(NVCC):
        return None
    hdrs = [os.path.join(REF_MAIN_SRC, f) for f in REF_MAIN_HEADERS]
    if force or _stale(REF_MAIN_BIN, srcs + hdrs):
        tmp = REF_MAIN_BIN + ".tmp"
        subprocess.run([NVCC, "-arch=sm_103a", "-O3", "-std=c++14", "--expt-relaxed-constexpr",
                        "-Xcompiler", "-Wno-format-truncation", "-w", "-o", tmp, *srcs, "-lcufft", "-lcudart", "-lm"],
                       check=True, cwd=REF_MAIN_SRC, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)
        os.replace(tmp, REF_MAIN_BIN)
    return REF_MAIN_BIN


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    if "--ref" in sys.argv:
        print(build_ref(force="--force" in sys.argv))
        print(build_ref_checkpoint(force="--force" in sys.argv))
        print(build_ref_kernels(force="--force" in sys.argv))
    if "--ref-main" in sys.argv:
        print(build_ref_main(force="--force" in sys.argv))
