"""Build recipe of liblulesh_gb300.so (sm_103a CUDA kernels + C ABI).

Compiles every translation unit in parallel with one -gencode and links a
shared library into lulesh.jl_gb300/lib/. The host setup file is compiled
without FMA contraction so the mesh matches the reference bit for bit.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "liblulesh_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + os.path.join(HERE, "..", "include")]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblulesh_gb300")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(verbose=False, defines=(), lib=LIB):
    """Builds the library at `lib` (objects in a _build folder beside it
    unless it is the in-tree default). `defines` adds -D macros, e.g.
    ("LULESH_CHECK",) for the index-checked debug build."""
    nvcc = _nvcc()
    obj = OBJ if lib == LIB else os.path.join(os.path.dirname(os.path.abspath(lib)), "_build")
    os.makedirs(obj, exist_ok=True)
    os.makedirs(os.path.dirname(os.path.abspath(lib)), exist_ok=True)
    dflags = ["-D" + m for m in defines]
    cu, cpp = _sources()
    jobs = []
    for f in cu:
        o = os.path.join(obj, f + ".o")
        jobs.append([nvcc] + ARCH + NVCC_FLAGS + dflags + ["-c", os.path.join(CSRC, f), "-o", o])
    for f in cpp:
        o = os.path.join(obj, f + ".o")
        jobs.append([os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off"] + dflags +
                    ["-c", os.path.join(CSRC, f), "-o", o])
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        for msg in ex.map(_run, jobs):
            if verbose and msg:
                print(msg)
    objs = [os.path.join(obj, f + ".o") for f in cu + cpp]
    _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
