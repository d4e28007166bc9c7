"""Build libsgpp_gb300.so in-tree with nvcc for sm_103a (GB300).

    python -m sgpp_gb300.build            # or: import sgpp_gb300.build as b; b.build()

Translation units are compiled in parallel into sgpp_gb300/_build/ and linked into
sgpp_gb300/libsgpp_gb300.so (a plain C-ABI shared library; no torch types).
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsgpp_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3,-fvisibility=hidden",
              "-I" + os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-Wall",
             "-I" + os.path.join(ROOT, "include")]

CU_SOURCES = ["sgmev.cu", "dense_mod.cu", "peak.cu", "noalloc.cu", "batch.cu", "subspace.cu",
              "subspace_mat.cu", "devmem.cu", "fitter.cu", "block_tc.cu"]
CPP_SOURCES = ["grid.cpp", "datasets.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources_newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]
    return hs


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile every translation unit (parallel) and link the shared library. Returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if ptxas_info or _sources_newer(o, [s] + headers):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _sources_newer(o, [s] + headers):
            jobs.append(["g++", *CXX_FLAGS, "-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stdout + r.stderr

    logs = []
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
            logs = list(ex.map(run, jobs))
    if jobs or _sources_newer(LIB, objs):
        link = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static"]
        run(link)
    if ptxas_info:
        for lg in logs:
            sys.stdout.write(lg)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
    print(LIB)
