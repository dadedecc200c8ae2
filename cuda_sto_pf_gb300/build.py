"""In-tree build of the pfgb CUDA library and the main_cuda host executable.

    python -m cuda_sto_pf_gb300.build          # incremental
    python -m cuda_sto_pf_gb300.build --force

Outputs (git-ignored) in cuda_sto_pf_gb300/_build/:
  libpfgb.so   -- the C-ABI library (include/pfgb.h), sm_103a kernels
  main_cuda    -- the drop-in CLI (host C++ above the C ABI)

Translation units are compiled in parallel; one -gencode (sm_103a).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libpfgb.so")
EXE = os.path.join(BUILD, "main_cuda")
INCLUDE = os.path.join(REPO, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
if not os.path.exists(NVCC):
    NVCC = shutil.which("nvcc") or "nvcc"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE,
              "--expt-relaxed-constexpr"] + ARCH

CU_SOURCES = ["solver.cu", "params.cu", "paramfile.cpp", "batch.cpp", "fno.cu", "checkpoint.cpp", "init.cu"]
HEADERS = ["common.cuh", "dfexp.cuh", "dfloat.cuh", "dft41_tc.cuh", "fft.cuh", "fft246.cuh", "physics.cuh", "rader41.cuh"]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src: str, force: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "pfgb.h")]
    if force or _newer(obj, deps):
        subprocess.run([NVCC, *NVCC_FLAGS, "-c", src, "-o", obj + ".tmp"], check=True)
        os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), srcs))
    if force or _newer(LIB, objs):
        subprocess.run([NVCC, *ARCH, "-shared", "-cudart", "shared", "-o", LIB + ".tmp", *objs],
                       check=True)
        os.replace(LIB + ".tmp", LIB)
    host_src = os.path.join(HOST, "main_cuda.cpp")
    if os.path.exists(host_src):
        host_deps = [host_src, LIB] + [os.path.join(HOST, f) for f in os.listdir(HOST)
                                        if f.endswith((".h", ".hpp", ".cpp"))]
        if force or _newer(EXE, host_deps):
            subprocess.run(["g++", "-std=c++17", "-O2", "-I", INCLUDE, "-I", HOST,
                            *[os.path.join(HOST, f) for f in sorted(os.listdir(HOST)) if f.endswith(".cpp")],
                            "-L", BUILD, "-lpfgb", "-Wl,-rpath,$ORIGIN", "-o", EXE + ".tmp"],
                           check=True)
            os.replace(EXE + ".tmp", EXE)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
