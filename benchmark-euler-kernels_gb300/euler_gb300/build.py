"""Build the CUDA library libeuler_gb300.so in-tree for sm_103a.

Each translation unit under ``csrc/`` is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked into
``benchmark-euler-kernels_gb300/lib/libeuler_gb300.so``.  Objects are reused
when they are newer than their sources and headers.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(REPO_ROOT, "include")
LIB_DIR = os.path.join(PKG_ROOT, "lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB_PATH = os.path.join(LIB_DIR, "libeuler_gb300.so")
APPS_DIR = os.path.join(PKG_ROOT, "apps")
APPS = ("euler_simulation", "euler_benchmarks")
APP_INCLUDES = ["-I", INCLUDE, "-I", os.path.join(INCLUDE, "euler_operators"),
                "-I", os.path.join(INCLUDE, "euler_operators_kokkos")]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC] + ARCH


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found")


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile every csrc/*.cu and link the shared library; returns its path."""
    nvcc = nvcc_path()
    os.makedirs(OBJ_DIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
                     + glob.glob(os.path.join(INCLUDE, "*.h")))
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *NVCC_FLAGS, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if jobs or force or _stale(LIB_PATH, objs):
        run([nvcc, "-shared", *ARCH, "-o", LIB_PATH, *objs])
    # host applications over the drop-in headers, linked against the library
    app_headers = headers + sorted(glob.glob(os.path.join(INCLUDE, "euler_operators", "*.hpp")) +
                                   glob.glob(os.path.join(INCLUDE, "euler_operators_kokkos", "*.hpp")))
    app_jobs = []
    for app in APPS:
        src = os.path.join(APPS_DIR, app + ".cpp")
        exe = os.path.join(LIB_DIR, app)
        if force or _stale(exe, [src, LIB_PATH] + app_headers):
            app_jobs.append([nvcc, "-std=c++20", "-O2", *APP_INCLUDES, src, "-o", exe, "-L", LIB_DIR, "-leuler_gb300",
                             "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(app_jobs))) as ex:
        list(ex.map(run, app_jobs))
    return LIB_PATH


def app_path(name: str) -> str:
    """Path of a built host application (euler_simulation, euler_benchmarks)."""
    return os.path.join(LIB_DIR, name)


if __name__ == "__main__":
    print(build(verbose=True))
