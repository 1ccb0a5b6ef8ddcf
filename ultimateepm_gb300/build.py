"""In-tree build of the native libraries (nvcc for sm_103a + g++), no cmake.

    python -m ultimateepm_gb300.build        # builds lib/libuepm_gb300.so and lib/libuepm_epp.so

Translation units compile in parallel; only changed sources are rebuilt.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
ADAPTER = os.path.join(PKG, "adapter")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libuepm_gb300.so")
EPP_LIB = os.path.join(OUT, "libuepm_epp.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-Xcompiler",
              "-ffp-contract=off",
              "--extended-lambda", "-I" + INCLUDE, "-I" + CSRC]
# assemble.cu mirrors the reference's operand order and rounding: no FMA contraction there.
PER_FILE = {"assemble.cu": ["--fmad=false"]}
# Host code: no FMA contraction, so the k-paths and the other host results are the same bits on
# x86 and Arm (gcc contracts a * b + c into one fma by default where the target has one).
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC]

CU_SOURCES = ["assemble.cu", "tridiag.cu", "tridiag_reg.cu", "tridiag_cluster.cu", "tridiag_blocked.cu", "tridiag_eig.cu", "backtransform.cu", "refine.cu", "refine_tc.cu", "capi.cu", "batch.cu", "server.cu", "star.cu", "peak.cu",
              "noalloc.cu", "dielectric.cu"]
CXX_SOURCES = ["host.cpp"]


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build ultimateepm_gb300")
    return p


def _cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _compile(src, verbose):
    base = os.path.basename(src)
    obj = os.path.join(OBJ, base + ".o")
    if not _stale(obj, [src] + _headers()):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *PER_FILE.get(base, []), "-c", src, "-o", obj]
    else:
        cmd = ["g++", *CXX_FLAGS, "-I" + os.path.join(_cuda_home(), "include"), "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {base}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = [os.path.join(CSRC, f) for f in CU_SOURCES + CXX_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if _stale(LIB, objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    # C++ adapter: the reference's uepm::pseudopotential classes over the C ABI
    if os.path.isdir(ADAPTER):
        asrcs = sorted(os.path.join(ADAPTER, f) for f in os.listdir(ADAPTER) if f.endswith(".cpp"))
        ahdrs = [os.path.join(INCLUDE, "uepm", f) for f in os.listdir(os.path.join(INCLUDE, "uepm"))] \
            if os.path.isdir(os.path.join(INCLUDE, "uepm")) else []
        if asrcs and _stale(EPP_LIB, asrcs + ahdrs + [LIB]):
            cmd = ["g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-Wall", "-ffp-contract=off", "-I" + INCLUDE,
                   "-I" + os.path.join(INCLUDE, "uepm"), *asrcs, "-o", EPP_LIB,
                   "-L" + OUT, "-luepm_gb300", "-Wl,-rpath,$ORIGIN"]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"adapter build failed\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
