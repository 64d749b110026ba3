"""Build recipe for libpd_gb300.so (sm_103a).

Compiles the CUDA translation units with nvcc and the host C++ with g++, in
parallel, into ``sci-solver_peridynamic_gb300/_build/`` and links
``sci-solver_peridynamic_gb300/libpd_gb300.so``.  Rebuilds only when a source
or header changed.  No cmake; one -gencode.

    python sci-solver_peridynamic_gb300/build.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpd_gb300.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["step.cu", "bonds.cu", "noalloc.cu", "mlp.cu", "mlp_tc.cu", "warmstart.cu", "batch.cu", "tiles.cu", "mesh_fill.cu", "contact.cu", "history.cu", "lattice.cu", "sph_coupling.cu"]
# per-file nvcc flags (none at present)
CU_EXTRA = {}
CPP_SOURCES = ["engine.cpp", "capi.cpp", "params.cpp", "batch.cpp", "dataio.cpp", "scene.cpp"]


def _sources_digest() -> str:
    h = hashlib.sha256()
    files = sorted(os.listdir(CSRC)) + ["../build.py"]
    for f in files:
        p = os.path.join(CSRC, f)
        if os.path.isfile(p):
            h.update(f.encode())
            with open(p, "rb") as fh:
                h.update(fh.read())
    for f in sorted(os.listdir(INCLUDE)):
        with open(os.path.join(INCLUDE, f), "rb") as fh:
            h.update(f.encode())
            h.update(fh.read())
    h.update(" ".join(ARCH).encode())
    return h.hexdigest()


def _compile(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link libpd_gb300.so if needed; returns its path."""
    digest = _sources_digest()
    stamp = os.path.join(BUILD, "digest")
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == digest:
                return LIB
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        jobs.append([NVCC, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off",
                     *CU_EXTRA.get(src, []), "-diag-suppress", "1444", "-I", INCLUDE, "-I", CSRC, "-c",
                     os.path.join(CSRC, src), "-o", obj])
    cxx = os.environ.get("CXX", "g++")
    for src in CPP_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        jobs.append([cxx, "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-I", INCLUDE, "-I", CSRC,
                     "-I", os.path.join(CUDA_HOME, "include"), "-c", os.path.join(CSRC, src), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_compile, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB + ".tmp"
    _compile([NVCC, "-shared", *ARCH, "-o", tmp, *objs, "-lpthread", "-ldl", "-lrt"])
    shutil.move(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
