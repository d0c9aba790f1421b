"""Builds libRobotecGPULidar.so in-tree (robotecgpulidar_gb300/_build) for sm_103a.

CUDA sources are compiled with nvcc (-gencode arch=compute_103a,code=sm_103a -lineinfo), host C++ with
g++, all translation units in parallel, then linked into one shared library whose exported symbols are
exactly the RGL_API functions of include/rgl/api. Host code is compiled with -ffp-contract=off so the
float math that builds rays and transforms evaluates identically on x86_64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libRobotecGPULidar.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _headers():
    out = []
    for d in (CSRC, os.path.join(INCLUDE, "rgl", "api"), os.path.join(INCLUDE, "rgl", "api", "extensions")):
        out += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".hpp", ".h"))]
    return out


def _stale(obj: str, src: str, headers) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src, *headers])


def build(verbose: bool = False, jobs: int | None = None) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = _headers()
    inc = ["-I", INCLUDE, "-I", CSRC]
    host_flags = ["-fPIC", "-fvisibility=hidden", "-ffp-contract=off"]
    cmds = []
    objs = []
    for f in sorted(os.listdir(CSRC)):
        src = os.path.join(CSRC, f)
        if f.endswith(".cu"):
            obj = os.path.join(OUT_DIR, f + ".o")
            cmd = [nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", ",".join(host_flags), *inc, "-c", src,
                   "-o", obj]
        elif f.endswith(".cpp"):
            obj = os.path.join(OUT_DIR, f + ".o")
            cmd = ["g++", "-std=c++17", "-O2", *host_flags, "-I", os.path.join(cuda, "include"), *inc, "-c", src,
                   "-o", obj]
        else:
            continue
        objs.append(obj)
        if _stale(obj, src, headers):
            cmds.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, cmds))
    if cmds or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        link = [nvcc, "-shared", *ARCH, "-o", LIB, *objs, "-lpthread"]
        run(link)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
