"""In-tree build of libcmsl_gb.so for sm_103a (nvcc only, no cmake).

    python -m cmsl_gb300.build
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libcmsl_gb.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CUDA_SOURCES = ["engine.cu", "noalloc.cu", "adjoint.cu", "grains.cu"]
HOST_SOURCES = ["formats.cpp"]
HEADERS = ["cmsl_dev.cuh", "dfloat.cuh", "kernels.cuh", "pcg_persist.cuh", "spectral.cuh", "stencil32.cuh",
           "stencil_tma.cuh", "tma.cuh",
           "engine.h"]
OBJDIR = os.path.join(HERE, "_build")


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


CLI = os.path.join(HERE, "cmsl_pe")
REFCOMPAT = os.path.join(HERE, "cmsl_refcompat.o")


def build_refcompat(verbose: bool = False, force: bool = False) -> str:
    """The object that defines the reference's Evolve/Depol_field entry points
    over its globals; link it with the reference's own objects and -lcmsl_gb."""
    src = os.path.join(CSRC, "refcompat.cu")
    deps = [src, os.path.join(ROOT, "include", "cmsl.h"), os.path.join(ROOT, "include", "cmsl_io.h")]
    if not force and not _stale(REFCOMPAT, deps):
        return REFCOMPAT
    cmd = [nvcc(), ARCH, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
           "-I" + os.path.join(ROOT, "include"),
           "-c", src, "-o", REFCOMPAT + ".tmp"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(REFCOMPAT + ".tmp", REFCOMPAT)
    return REFCOMPAT


def build_cli(verbose: bool = False, force: bool = False) -> str:
    """The campaign driver executable (cmsl_pe), linked against libcmsl_gb.so."""
    src = os.path.join(CSRC, "cmsl_pe.cpp")
    deps = [src, OUT, os.path.join(ROOT, "include", "cmsl.h"), os.path.join(ROOT, "include", "cmsl_io.h")]
    if not force and not _stale(CLI, deps):
        return CLI
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-ffp-contract=off",
           "-I" + os.path.join(ROOT, "include"), src, "-L" + HERE, "-lcmsl_gb", "-Wl,-rpath,$ORIGIN",
           "-o", CLI + ".tmp"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(CLI + ".tmp", CLI)
    return CLI


def build(verbose: bool = False, force: bool = False) -> str:
    """Compiles every translation unit to an object in parallel (one nvcc per
    source), then links libcmsl_gb.so."""
    srcs = [os.path.join(CSRC, s) for s in CUDA_SOURCES + HOST_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    deps = srcs + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "cmsl.h"),
                                                             os.path.join(ROOT, "include", "cmsl_io.h")]
    if not force and not _stale(OUT, deps):
        return OUT
    os.makedirs(OBJDIR, exist_ok=True)
    common = [nvcc(), ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    objs, procs = [], []
    for src in srcs:
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        objs.append(obj)
        cmd = common + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((cmd, subprocess.Popen(cmd)))
    for cmd, p in procs:
        if p.wait() != 0:
            raise subprocess.CalledProcessError(p.returncode, cmd)
    tmp = OUT + ".tmp"
    cmd = [nvcc(), ARCH, "-shared", "-o", tmp] + objs + ["-lcudart"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


def build_all(verbose: bool = False, force: bool = False) -> str:
    out = build(verbose=verbose, force=force)
    build_cli(verbose=verbose, force=force)
    build_refcompat(verbose=verbose, force=force)
    return out


if __name__ == "__main__":
    print(build_all(verbose=True, force="--force" in sys.argv))
