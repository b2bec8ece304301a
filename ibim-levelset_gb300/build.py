"""Build libibim_gb300.so (sm_103a) in-tree with nvcc: one translation unit per process, in parallel."""

from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libibim_gb300.so")
SOURCES = ["levelset.cu", "tree.cpp", "fmm.cu", "fmm_mixed.cu", "near_ff.cu", "m2l_tc.cu", "solve.cu", "capi.cu",
           "server.cpp", "batch.cu", "tuning.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
OPENMP_CU = {"fmm.cu", "fmm_mixed.cu"}  # CUDA files whose host code (plan building) uses OpenMP
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-Xcompiler", "-Wno-unused-function", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _obj(src: str) -> str:
    return os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")


def _compile(src: str, verbose: bool) -> str:
    path = os.path.join(CSRC, src)
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS]
    if src.endswith(".cpp"):
        cmd += ["-x", "cu", "-Xcompiler", "-fopenmp"]
    elif src in OPENMP_CU:
        cmd += ["-Xcompiler", "-fopenmp"]
    cmd += ["-c", path, "-o", _obj(src)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, os.pardir, "include", "ibim.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA translation unit for sm_103a and link the shared library."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        logs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if verbose:
        for s, log in zip(SOURCES, logs):
            print(f"== {s}\n{log}")
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *[_obj(s) for s in SOURCES], "-lcudart", "-lgomp", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
