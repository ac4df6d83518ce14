"""Builds the engine shared library in-tree with nvcc for sm_103a.

    python -m fideslib_gb300.build            # -> fideslib_gb300/_lib/libfideslib_gb300.so

Translation units are compiled in parallel and linked with `nvcc -shared`; the CUDA runtime is linked
statically so the library only needs the driver at run time.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libfideslib_gb300.so"
SOURCES = ["ntt.cu", "kernels.cu", "engine.cu", "capi.cu", "noalloc.cu", "server.cu", "poly_eval.cu", "bootstrap.cu",
           "encode.cu", "autoscale.cu", "rawfile.cu", "probe.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-Wno-deprecated-gpu-targets"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def lib_path() -> str:
    return os.path.join(OUT_DIR, LIB_NAME)


def _needs_build(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "fideslib_gb300.h"))
    cc = nvcc()
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src + ".o")
        if _needs_build(o, [s] + headers):
            cmd = [cc, *ARCH, *FLAGS, *(extra or []), "-c", s, "-o", o]
            jobs.append(cmd)
    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(OBJ_DIR, s + ".o") for s in SOURCES]
    lib = lib_path()
    if jobs or not os.path.exists(lib):
        cmd = [cc, *ARCH, "-shared", "-o", lib, *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
