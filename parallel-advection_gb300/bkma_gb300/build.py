"""In-tree build of libbkma_gb300.so (nvcc, sm_103a only) and of the C++
host applications (advection / conv1d drivers with the reference's .ini
interface).

Objects go to parallel-advection_gb300/_build/, the library to
parallel-advection_gb300/libbkma_gb300.so. Translation units compile in
parallel; a unit is rebuilt when it or any header is newer than its object.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
HOST = os.path.join(PKG_ROOT, "host")
INCLUDE = os.path.join(REPO_ROOT, "include")
BUILD = os.path.join(PKG_ROOT, "_build")
LIB = os.path.join(PKG_ROOT, "libbkma_gb300.so")
BIN = os.path.join(PKG_ROOT, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest(paths) -> float:
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build_library(force: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    hdr_time = _newest(headers)
    nv = nvcc()
    jobs_todo = []
    objs = []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(
                os.path.getmtime(src), hdr_time):
            jobs_todo.append([nv] + NVCC_FLAGS + ["-c", src, "-o", obj])
    if jobs_todo:
        with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs_todo))
    if force or jobs_todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        tmp = LIB + ".tmp"
        _run([nv] + ARCH + ["-shared", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    return LIB


def build_host_apps(force: bool = False) -> list[str]:
    """The C++ drivers that mirror src/advection.cpp and src/conv1d.cpp over the C ABI."""
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    if not srcs:
        return []
    os.makedirs(BIN, exist_ok=True)
    common = [s for s in srcs if not os.path.basename(s).startswith("app_")]
    apps = [s for s in srcs if os.path.basename(s).startswith("app_")]
    hdrs = glob.glob(os.path.join(HOST, "*.hpp")) + [os.path.join(INCLUDE, "bkma_gb300.h")]
    out = []
    cxx = os.environ.get("CXX", "g++")
    cuda_root = os.path.dirname(os.path.dirname(nvcc()))
    cuda_inc = os.path.join(cuda_root, "include")
    cuda_lib = os.path.join(cuda_root, "lib64")
    for app in apps:
        name = os.path.basename(app)[len("app_"):-len(".cpp")]
        exe = os.path.join(BIN, name)
        deps = [app] + common + hdrs + [LIB]
        if force or not os.path.exists(exe) or os.path.getmtime(exe) < _newest(deps):
            _run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", INCLUDE, "-I", HOST,
                  "-I", cuda_inc, app] + common +
                 ["-o", exe, "-L", PKG_ROOT, "-lbkma_gb300", "-L", cuda_lib, "-lcudart",
                  "-Wl,-rpath,$ORIGIN/..", "-Wl,-rpath," + cuda_lib])
        out.append(exe)
    return out


if __name__ == "__main__":
    print(build_library())
    print(build_host_apps())
