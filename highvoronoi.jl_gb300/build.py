"""Builds libhvgpu.so (sm_103a) in-tree: one nvcc job per translation unit, in
parallel, then a shared-library link.  No cmake, no torch extension: the
product is a plain C-ABI library (include/hvgpu.h)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libhvgpu.so")
SOURCES = ["hv_prep.cu", "hv_search.cu", "hv_search_d2.cu", "hv_search_d3.cu", "hv_search_d4.cu",
           "hv_search_d5.cu", "hv_search_d6.cu", "hv_post.cu", "hv_integrate.cu", "hv_poly.cu", "hv_api.cu", "hv_server.cpp", "hv_noalloc.cu",
           "hv_domain.cu", "hv_periodic.cu", "hv_quad.cu", "hv_degen.cu", "hv_polyflag.cu", "hv_polylat.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + [
        os.path.join(ROOT, "include", "hvgpu.h")]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    hdrs = _headers()
    nvcc = _nvcc()
    jobs = []
    for s in srcs:
        obj = os.path.join(OUT, os.path.splitext(s)[0] + ".o")
        if force or _stale(obj, [os.path.join(CSRC, s)] + hdrs):
            cmd = [nvcc, *FLAGS, *ARCH, *extra_flags, "-c", os.path.join(CSRC, s), "-o", obj]
            jobs.append((s, cmd))

    def run(job):
        name, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return name, r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for name, r in ex.map(run, jobs):
            if verbose and r.stderr:
                sys.stderr.write(r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr}")
    objs = [os.path.join(OUT, os.path.splitext(s)[0] + ".o") for s in srcs]
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, "-shared", *ARCH, "-o", LIB, *objs, "-Xcompiler", "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
