"""Build libdeo.so in-tree for sm_103a (nvcc + g++, two translation units
compiled in parallel; no cmake).  Output: diffeqoperators.jl_gb300/libdeo.so"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdeo.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = {
    "deo_kernels.o": ("nvcc", "deo_kernels.cu"),
    "deo_tma.o": ("nvcc", "deo_tma.cu"),
    "deo_vec.o": ("nvcc", "deo_vec.cu"),
    "deo_concretize.o": ("nvcc", "deo_concretize.cu"),
    "deo_shell.o": ("nvcc", "deo_shell.cu"),
    "deo_static.o": ("nvcc", "deo_static.cu"),
    "deo_vector.o": ("nvcc", "deo_vector.cu"),
    "deo_solve.o": ("nvcc", "deo_solve.cu"),
    "deo_host.o": ("cxx", "deo_host.cpp"),
    "deo_serve.o": ("cxx", "deo_serve.cpp"),
}


def _cmd(kind: str, src: str, obj: str, verbose_ptxas: bool) -> list[str]:
    inc = ["-I", os.path.join(HERE, "..", "include"), "-I", CSRC]
    if kind == "nvcc":
        c = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-c", src,
             "-o", obj, *inc]
        if verbose_ptxas:
            c += ["-Xptxas", "-v"]
        return c
    # -ffp-contract=off: host arithmetic (Fornberg weights, BC maps) rounds every
    # product and sum as the reference does; GCC fuses a*b+c on Arm otherwise.
    return ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-c", src, "-o", obj, *inc,
            "-I", os.path.join(CUDA_HOME, "include")]


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src, os.path.join(CSRC, "deo_internal.h"), os.path.join(CSRC, "deo_eval.cuh"),
            os.path.join(CSRC, "deo_rows.cuh"), os.path.join(CSRC, "deo_ptx.cuh"), os.path.join(CSRC, "deo_fx.cuh"),
            os.path.join(CSRC, "deo_bfx.cuh"), os.path.join(CSRC, "deo_lap.cuh"),
            os.path.join(HERE, "..", "include", "deo.h"),
            os.path.abspath(__file__)]
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    for obj, (kind, src) in SOURCES.items():
        o = os.path.join(BUILD, obj)
        s = os.path.join(CSRC, src)
        if force or verbose_ptxas or _stale(o, s):
            jobs.append(_cmd(kind, s, o, verbose_ptxas))
    if jobs:
        with cf.ThreadPoolExecutor(len(jobs)) as ex:
            for r in ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs):
                if r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                    raise RuntimeError("libdeo build failed: " + " ".join(r.args))
                if verbose_ptxas and r.stderr:
                    sys.stderr.write(r.stderr)
    objs = [os.path.join(BUILD, o) for o in SOURCES]
    if jobs or not os.path.exists(LIB):
        link = [NVCC, *ARCH, "-shared", "-cudart", "shared", "-o", LIB, *objs]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("libdeo link failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
