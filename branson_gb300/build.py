"""Build the sm_103a library in-tree: branson_gb300/_build/libbranson_gb300.so.

Each translation unit under csrc/ is compiled by nvcc in parallel for
``sm_103a`` only, without FMA contraction (``-fmad=false``) so that FP64
expressions round like the upstream C++ built without contraction, and then
linked into one shared library exposing the C ABI of include/branson_gb300.h.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libbranson_gb300.so")
SOURCES = ("bgs_api.cu", "bgs_mesh.cu", "bgs_source.cu", "bgs_transport.cu", "bgs_event.cu", "bgs_noalloc.cu",
           "bgs_adjoint.cu", "bgs_adjoint_api.cu", "bgs_batch.cu", "bgs_batch_api.cu", "bgs_comb.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr",
              "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build branson_gb300")


def _headers_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    paths.append(os.path.join(ROOT, "include", "branson_gb300.h"))
    return max(os.path.getmtime(p) for p in paths)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile (if stale) and return the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    hdr = _headers_mtime()
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        stale = force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr)
        if stale or ptxas_info:
            cmd = [cc, *ARCH, *NVCC_FLAGS, "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append((src, cmd))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): src for src, cmd in jobs}
            for fut, src in futs.items():
                r = fut.result()
                if verbose or ptxas_info:
                    sys.stdout.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if force or jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(cc))), "lib64")
        cmd = [cc, *ARCH, "-shared", "-cudart", "shared", "-o", LIB, *objs,
               "-Xlinker", f"-rpath,{cuda_lib}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
