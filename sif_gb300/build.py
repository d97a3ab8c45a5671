"""Builds libsif_gb300.so in-tree from sif_gb300/csrc with nvcc for sm_103a.

Each translation unit compiles in its own nvcc process, in parallel, then one
link. Host code is compiled with -ffp-contract=off: the per-rung constants the
kernels receive are float expressions that must round as the reference's.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsif_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
UNITS = ["scan", "cic", "mesh", "smooth", "finder", "engine", "api", "noalloc", "hostpool", "adjoint",
         "checkpoint", "mirror", "survey"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _flags():
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off",
            "-I" + os.path.join(HERE, "..", "include")]


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "sif_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit):
    src = os.path.join(CSRC, unit + ".cu")
    obj = os.path.join(BUILD, unit + ".o")
    if not _stale(obj, src):
        return None
    cmd = [nvcc()] + _flags() + ["-c", src, "-o", obj]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        return f"{unit}: {' '.join(cmd)}\n{out.stdout}{out.stderr}"
    return None


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        errors = [e for e in ex.map(_compile, UNITS) if e]
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    objs = [os.path.join(BUILD, u + ".o") for u in UNITS]
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", LIB] + objs + ["-lcufft", "-lgomp"]
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + out.stdout + out.stderr)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
