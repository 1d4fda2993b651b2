"""Compile libcpm_gpu.so in-tree for sm_103a (GB300).

Usage: ``python cpm-rust_gb300/build.py [--force]``. Translation units are
compiled in parallel with nvcc (CUDA) and g++ (host C++), then linked into
``cpm-rust_gb300/lib/libcpm_gpu.so`` with the CUDA runtime linked statically
(so the library does not depend on which libcudart a host process loads).
Host code is built with -ffp-contract=off: the readouts restate the
reference's f64 formulas and must not pick up fused multiply-adds.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libcpm_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["cpm_kernels.cu", "cpm_resident.cu", "cpm_resident_modes.cu", "cpm_tiled.cu", "cpm_tiled_odd.cu",
              "cpm_tiled_modes.cu", "cpm_tiled_modes_odd.cu", "cpm_init_device.cu",
              "cpm_noalloc.cu", "cpm_readout.cu"]
CPP_SOURCES = ["cpm_config.cpp", "cpm_init.cpp", "cpm_engine.cpp", "cpm_serve.cpp", "cpm_capi.cpp"]


def _cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: the GB300 engine needs the CUDA toolkit to build")


def _newest_input() -> float:
    t = 0.0
    for d in (CSRC, os.path.join(os.path.dirname(HERE), "include")):
        for f in os.listdir(d):
            t = max(t, os.path.getmtime(os.path.join(d, f)))
    return max(t, os.path.getmtime(__file__))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input():
        return LIB
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    inc = ["-I", CSRC, "-I", os.path.join(cuda, "include")]
    jobs = []
    for src in CU_SOURCES:
        obj = os.path.join(OBJDIR, src + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
               *inc, "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((cmd, obj))
    for src in CPP_SOURCES:
        obj = os.path.join(OBJDIR, src + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread",
               *inc, "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((cmd, obj))

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        return p.stderr

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, [c for c, _ in jobs]))
    tmp = LIB + ".tmp"
    link = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *[o for _, o in jobs],
            "-Xcompiler", "-pthread", "-lpthread", "-ldl", "-lrt"]
    run(link)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
