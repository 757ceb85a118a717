"""In-tree build of libsimall_gpu.so for sm_103a (nvcc, no cmake).

Every CUDA translation unit is compiled for `-gencode arch=compute_103a,
code=sm_103a` in parallel and linked into simall_gb300/lib/libsimall_gpu.so.
Host C++ is compiled with -ffp-contract=off: the mesh generator must produce
the reference's geometry bit for bit, and gcc on aarch64 would otherwise fuse
multiply-adds.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libsimall_gpu.so")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _deps() -> list[str]:
    return glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(obj: str, src: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile (incrementally) and link libsimall_gpu.so; returns its path."""
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    deps = _deps()
    common = ["-O3", "-std=c++17", f"-I{INCLUDE}", f"-I{CSRC}", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fvisibility=default"]
    jobs = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if not _stale(obj, src, deps):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc, ARCH, "-lineinfo", *common, "-c", src, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
        else:
            cmd = [nvcc, "-x", "c++", *common, "-c", src, "-o", obj]
        jobs.append((src, cmd))
    procs = []
    for src, cmd in jobs:
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if out and (verbose or p.returncode or ptxas_info):
            sys.stdout.write(out)
        if p.returncode:
            failed.append(src)
    if failed:
        raise RuntimeError("nvcc failed for: " + ", ".join(os.path.basename(f) for f in failed))
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        # the shared CUDA runtime: a process that also loads PyTorch then has
        # a single runtime instance (same SONAME) instead of two
        cudalib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(shutil.which(nvcc) or nvcc))),
                               "lib64")
        cmd = [nvcc, ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs, f"-Xlinker=-rpath,{cudalib}",
               "-lrt", "-lpthread", "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
