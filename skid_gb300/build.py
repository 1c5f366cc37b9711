"""Build libskidgpu (sm_103a) and the `skid` command-line tool in-tree.

    python -m skid_gb300.build          # library + CLI
    python -m skid_gb300.build --lib    # library only

Each CUDA translation unit is compiled in parallel with one -gencode for
sm_103a; the objects are linked with nvcc into skid_gb300/lib/libskidgpu.so.
The CLI (C) links that library.  No CMake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
OBJDIR = os.path.join(PKG, "lib", "obj")
LIB = os.path.join(LIBDIR, "libskidgpu.so")
CLI = os.path.join(BINDIR, "skid")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "skid_gpu.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_lib(force: bool = False, verbose: bool = False, extra=()) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    srcs = _sources()
    hdrs = _headers()
    objs = [os.path.join(OBJDIR, os.path.basename(s)[:-3] + ".o") for s in srcs]
    cc = nvcc()

    def one(src, obj):
        if not force and not _stale(obj, [src] + hdrs):
            return None
        cmd = [cc, *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda a: one(*a), zip(srcs, objs)))
    if force or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def build_cli(force: bool = False) -> str | None:
    if not os.path.isdir(HOST):
        return None
    srcs = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".c"))
    if not srcs:
        return None
    os.makedirs(BINDIR, exist_ok=True)
    deps = srcs + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")] + [LIB]
    if force or _stale(CLI, deps):
        tmp = CLI + f".tmp{os.getpid()}"
        cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off", "-Wall",
               "-I" + os.path.join(ROOT, "include"), "-o", tmp, *srcs, "-L" + LIBDIR, "-lskidgpu",
               "-Wl,-rpath,$ORIGIN/../lib", "-lm", "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"CLI build failed:\n{r.stderr}")
        os.replace(tmp, CLI)
    return CLI


def build(force: bool = False, verbose: bool = False) -> str:
    lib = build_lib(force=force, verbose=verbose)
    build_cli(force=force)
    return lib


if __name__ == "__main__":
    a = sys.argv[1:]
    if "--lib" in a:
        print(build_lib(force="-f" in a, verbose=True))
    else:
        print(build(force="-f" in a, verbose=True))
