"""Builds libkite_gb300.so in-tree: the sm_103a kernels, the engine and the kite C API.

nvcc compiles the CUDA translation units for sm_103a only and g++ the host ones, in parallel;
the link uses nvcc with the static CUDA runtime.  A stamp of the sources and flags skips
rebuilds that would produce the same library.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libkite_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC", "-Xptxas", "-O3"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"]


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    hdr = sorted(f for f in os.listdir(CSRC) if f.endswith((".h", ".cuh")))
    return cu, cpp, hdr


def _stamp(files) -> str:
    h = hashlib.sha256()
    for f in files:
        with open(f, "rb") as fh:
            h.update(f.encode())
            h.update(fh.read())
    h.update(" ".join(NVCC_FLAGS + CXX_FLAGS).encode())
    return h.hexdigest()


def build_library(force: bool = False, verbose: bool = False) -> str:
    """Compile and link the library if needed; returns its path."""
    cu, cpp, hdr = _sources()
    inc_files = [os.path.join(INCLUDE, f) for f in sorted(os.listdir(INCLUDE)) if f.endswith(".h")]
    files = [os.path.join(CSRC, f) for f in cu + cpp + hdr] + inc_files
    stamp = _stamp(files)
    stamp_path = os.path.join(BUILD, "stamp")
    if not force and os.path.exists(LIB) and os.path.exists(stamp_path):
        with open(stamp_path) as fh:
            if fh.read().strip() == stamp:
                return LIB
    os.makedirs(BUILD, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    cxx = os.environ.get("CXX", "g++")
    jobs = []
    for f in cu:
        obj = os.path.join(BUILD, f + ".o")
        jobs.append([nvcc] + NVCC_FLAGS + ["-I", INCLUDE, "-c", os.path.join(CSRC, f), "-o", obj])
    for f in cpp:
        obj = os.path.join(BUILD, f + ".o")
        jobs.append([cxx] + CXX_FLAGS + ["-I", INCLUDE, "-I", os.path.join(cuda, "include"),
                                         "-c", os.path.join(CSRC, f), "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, f + ".o") for f in cu + cpp]
    tmp = LIB + ".tmp"
    run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread", "-lrt", "-ldl"])
    os.replace(tmp, LIB)
    with open(stamp_path, "w") as fh:
        fh.write(stamp)
    return LIB


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
