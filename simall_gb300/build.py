"""In-tree build of libsimall_gpu.so for sm_103a (nvcc, no cmake).

Every CUDA translation unit is compiled for `-gencode arch=compute_103a,
code=sm_103a` in parallel and linked into simall_gb300/lib/libsimall_gpu.so.
Host C++ is compiled with -ffp-contract=off: the mesh generator must produce
the reference's geometry bit for bit, and gcc on aarch64 would otherwise fuse
multiply-adds.

An object is reused only when a key over its source, every header, the
compile command and the host (machine type, compiler version) equals the key
it was built with (lib/obj/keys.json); file times play no part, so objects
copied from another host or restored with new times are rebuilt.  Each build
writes lib/build_info.json: the host, and which objects it compiled and which
it reused.
"""
from __future__ import annotations

import glob
import hashlib
import json
import os
import platform
import shutil
import subprocess
import sys
import time

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


def _compiler_id(nvcc: str) -> str:
    try:
        return subprocess.run([nvcc, "--version"], capture_output=True, text=True).stdout.strip().splitlines()[-1]
    except (OSError, IndexError):
        return "unknown"


def _key(src: str, deps: list[str], cmd: list[str], host: str) -> str:
    h = hashlib.sha256()
    h.update(host.encode())
    h.update(" ".join(cmd).encode())
    for p in [src] + sorted(deps):
        h.update(p.encode())
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile what changed and link libsimall_gpu.so; returns its path."""
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    deps = _deps()
    host = f"{platform.machine()} {_compiler_id(nvcc)}"
    keys_path = os.path.join(OBJDIR, "keys.json")
    try:
        with open(keys_path) as f:
            old_keys = json.load(f)
        if old_keys.get("_host") != host:
            old_keys = {}
    except (OSError, ValueError):
        old_keys = {}
    new_keys = {"_host": host}
    reused = []
    common = ["-O3", "-std=c++17", f"-I{INCLUDE}", f"-I{CSRC}", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fvisibility=default"]
    jobs = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if src.endswith(".cu"):
            cmd = [nvcc, ARCH, "-lineinfo", *common, "-c", src, "-o", obj]
        else:
            cmd = [nvcc, "-x", "c++", *common, "-c", src, "-o", obj]
        key = _key(src, deps, cmd, host)
        new_keys[os.path.basename(src)] = key
        if os.path.exists(obj) and old_keys.get(os.path.basename(src)) == key and not ptxas_info:
            reused.append(os.path.basename(src))
            continue
        if ptxas_info and src.endswith(".cu"):
            cmd.insert(1, "-Xptxas=-v")
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
        with open(keys_path, "w") as f:  # the failed objects keep no key
            json.dump({k: v for k, v in new_keys.items() if k not in {os.path.basename(x) for x in failed}}, f)
        raise RuntimeError("nvcc failed for: " + ", ".join(os.path.basename(f) for f in failed))
    with open(keys_path, "w") as f:
        json.dump(new_keys, f)
    linked = False
    if jobs or not os.path.exists(LIB):
        linked = True
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
    with open(os.path.join(LIBDIR, "build_info.json"), "w") as f:
        json.dump({"host": host, "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
                   "compiled": sorted(os.path.basename(s_) for s_, _ in jobs), "reused": sorted(reused),
                   "linked": linked}, f, indent=1)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
