"""Build librheogpu.so in-tree: nvcc for sm_103a, one object per .cu in parallel."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
OUT = os.path.join(HERE, "librheogpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "rheogpu.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, extra=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    objs = []
    jobs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append([cc, *ARCH, *FLAGS, *extra, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        res = list(ex.map(lambda cmd: subprocess.run(cmd, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, res):
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    if jobs or not os.path.exists(OUT):
        link = [cc, *ARCH, "-shared", "-o", OUT, *objs, "-lcudart"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    build_host()
    return OUT


HOST = os.path.join(HERE, "host")
HOST_OUT = os.path.join(HERE, "librheogpu_host.so")


def build_host() -> str:
    """The C++ host mirror (host/rheogpu_host.cpp) as librheogpu_host.so,
    linked to librheogpu.so beside it."""
    src = os.path.join(HOST, "rheogpu_host.cpp")
    deps = [src, os.path.join(HOST, "rheogpu.hpp"), os.path.join(HERE, "..", "include", "rheogpu.h"), OUT]
    if os.path.exists(HOST_OUT) and all(os.path.getmtime(d) <= os.path.getmtime(HOST_OUT) for d in deps):
        return HOST_OUT
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler for the host library")
    cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-o", HOST_OUT, src, "-L" + HERE, "-lrheogpu",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("host library build failed")
    return HOST_OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
