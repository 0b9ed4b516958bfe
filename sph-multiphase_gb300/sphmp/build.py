"""Build libsphmp.so in-tree for sm_103a.

Compiles the CUDA translation units with nvcc (one -gencode, sm_103a) and the
host-only setup code with the host compiler, in parallel, and links a shared
library into sph-multiphase_gb300/sphmp/_lib/. No CMake; rebuilds only when a
source is newer than the library.
"""
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                 # sph-multiphase_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
LIB_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB_PATH = os.path.join(LIB_DIR, "libsphmp.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["sphmp_kernels.cu", "sphmp_api.cu", "sphmp_iisph.cu", "sphmp_noalloc.cu", "sphmp_mlp.cu",
                "sphmp_learned.cu"]
HOST_SOURCES = ["sphmp_host.cpp", "sphmp_io.cpp"]


def _nvcc():
    env = os.environ.get("NVCC")
    if env:
        return env
    for cand in ("/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found (set NVCC)")


def _sources():
    out = [os.path.join(CSRC, f) for f in CUDA_SOURCES + HOST_SOURCES]
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    out += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    out.append(os.path.abspath(__file__))
    return out


def up_to_date():
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False, extra_nvcc=()):
    """Compile and link libsphmp.so; returns its path."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = _nvcc()
    cxx = os.environ.get("CXX", "g++")
    common_inc = ["-I", INCLUDE, "-I", CSRC]
    jobs = []
    objs = []
    for f in CUDA_SOURCES:
        obj = os.path.join(OBJ_DIR, f + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", *common_inc, *extra_nvcc, "-c",
               os.path.join(CSRC, f), "-o", obj]
        jobs.append((f, cmd))
        objs.append(obj)
    for f in HOST_SOURCES:
        obj = os.path.join(OBJ_DIR, f + ".o")
        cmd = [cxx, "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall", *common_inc, "-c",
               os.path.join(CSRC, f), "-o", obj]
        jobs.append((f, cmd))
        objs.append(obj)
    procs = [(f, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for f, cmd in jobs]
    failed = []
    for f, cmd, p in procs:
        out, _ = p.communicate()
        if verbose and out.strip():
            print(out)
        if p.returncode != 0:
            failed.append((f, " ".join(cmd), out))
    if failed:
        msg = "\n".join(f"--- {f}\n{c}\n{o}" for f, c, o in failed)
        raise RuntimeError("libsphmp build failed:\n" + msg)
    tmp = LIB_PATH + ".tmp"
    subprocess.check_call([nvcc, *ARCH, "-shared", "-o", tmp, *objs])
    os.replace(tmp, LIB_PATH)
    if verbose:
        print("built", LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
