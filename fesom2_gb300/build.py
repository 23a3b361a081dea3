"""In-tree build of libfesom_gpu.so for sm_103a (nvcc + g++, no cmake).

``python -m fesom2_gb300.build`` or ``fesom2_gb300.build.build()``; the
translation units compile in parallel and the result lands in
``fesom2_gb300/_build/libfesom_gpu.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfesom_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                      "-Xptxas", "-warn-spills"]
UNITS = {
    # FP64 kernels: no FMA contraction, so the arithmetic matches the reference bit for bit
    "kernels_fp64.cu": ["--fmad=false"],
    "kernels_fp32.cu": [],
    "kernels_fp32_batched.cu": [],
    "capi.cu": [],
    # allocation-free vertical diffusion: FP64, same rounding as kernels_fp64.cu
    "vdiff_noalloc.cu": ["--fmad=false"],
    # tail of the tracer loop (decay, climatology relaxation, clamps): FP64, no contraction
    "kernels_tail.cu": ["--fmad=false"],
}
HOST_UNITS = ["mesh_prep.cpp"]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "fesom_gpu.h"))
    jobs = []
    objs = []
    for src, extra in UNITS.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + NVCC_COMMON + extra + ["-c", s, "-o", o])
    for src in HOST_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
