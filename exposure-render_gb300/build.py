"""Builds libexposurerender.so for sm_103a (nvcc, no cmake).

Translation units:
  er_render.cu, er_post.cu  reference-order kernels, --fmad=false so that the
                            GPU evaluates the same floating-point operations
                            as the reference's host build;
  er_runtime.cu             host runtime behind the C ABI, -ffp-contract=off
                            for the host arithmetic that feeds the kernels.
Each TU compiles in its own nvcc process (in parallel); objects and the
shared library go to exposure-render_gb300/_build/.
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
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libexposurerender.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
          "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

UNITS = {
    "er_render.cu": ["--fmad=false", "-Xptxas", "-v"],
    "er_post.cu": ["--fmad=false"],
    "er_volume.cu": ["--fmad=false"],
    "er_wavefront.cu": ["--fmad=false", "-Xptxas", "-v"],
    "er_medium.cu": ["--fmad=false", "-Xptxas", "-v"],
    "er_runtime.cu": [],
    "er_cxx_api.cpp": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str], verbose: bool) -> tuple[str, str]:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr if verbose else ""


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    jobs = {}
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        for src, extra in UNITS.items():
            obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
            if force or _stale(obj, [os.path.join(CSRC, src), *headers]):
                jobs[src] = ex.submit(_compile, src, extra, verbose)
        logs = {k: f.result() for k, f in jobs.items()}
    objs = [os.path.join(OUT, os.path.splitext(s)[0] + ".o") for s in UNITS]
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", LIB]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        for k, (_, log) in logs.items():
            if log:
                print(f"--- {k}\n{log}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
