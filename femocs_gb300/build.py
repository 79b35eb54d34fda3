"""In-tree build of the femocs_gb300 shared library (C++ host code + sm_103a CUDA kernels).

    python -m femocs_gb300.build          # builds femocs_gb300/_build/libfemocs_gb300.so

Every .cu file is compiled for sm_103a only; files named *_exact.cu are compiled with
-fmad=false because they reproduce the reference's floating-point operation order bit for
bit (cell location, interpolation, nodal-field recovery). Host C++ is compiled with
-ffp-contract=off for the same reason and so that x86 and Arm hosts agree.
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
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfemocs_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _sources():
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    return cpp, cu


def _headers_mtime() -> float:
    m = 0.0
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def _compile(cmd, src, obj, hdr_mtime, force):
    if not force and os.path.exists(obj):
        om = os.path.getmtime(obj)
        if om >= os.path.getmtime(src) and om >= hdr_mtime:
            return obj
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I", CSRC, "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include")]
    cpp, cu = _sources()
    hm = _headers_mtime()
    jobs = []
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f[:-4] + ".o")
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fopenmp", "-Wall",
               "-Wno-unused-function", *inc, "-c", src, "-o", obj]
        jobs.append((cmd, src, obj))
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f[:-3] + ".o")
        extra = ["-fmad=false"] if f.endswith("_exact.cu") else []
        cmd = [nvcc, *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp",
               "-Xptxas", "-warn-spills", *extra, *inc, "-c", src, "-o", obj]
        jobs.append((cmd, src, obj))
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda j: _compile(*j, hm, force), jobs))
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
