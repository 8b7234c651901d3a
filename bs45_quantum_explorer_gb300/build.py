"""In-tree build of libbsfh.so (sm_103a) and of the C++ lane binary.

Each .cu translation unit is compiled in parallel with
`nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`, then linked as a shared
library beside this file. No cmake, no torch extension machinery.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libbsfh.so")
BIN = os.path.join(PKG, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbsfh.so")
    return exe


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


# host translation units linked into the library (the cell algebra behind bs_cell_list and
# bs_ab_rows); the lane's main() is built separately as bin/bs_firsthit
LIB_HOST = ["celllist.cpp", "cell_capi.cpp"]
HOSTFLAGS = ["-O2", "-std=c++17", "-fPIC", "-pthread", f"-I{INCLUDE}"]


def build_library(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "bsfh.h"))
    host_headers = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
    jobs = []
    objs = []
    for src in _sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc()] + NVFLAGS + ["-c", src, "-o", obj])
    for name in LIB_HOST:
        src = os.path.join(HOST, name)
        obj = os.path.join(BUILD, "host_" + name[:-4] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, os.path.join(INCLUDE, "bsfh.h")] + host_headers):
            jobs.append(["g++"] + HOSTFLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
        if verbose and r.stderr:
            print(r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stderr}")
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stderr}")
    return LIB


def build_host(force=False):
    """Builds the drop-in lane binary bin/bs_firsthit (C++ host over libbsfh.so)."""
    srcs = [os.path.join(HOST, "firsthit_main.cpp")]
    os.makedirs(BIN, exist_ok=True)
    exe = os.path.join(BIN, "bs_firsthit")
    hdrs = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
    if force or _stale(exe, srcs + hdrs + [LIB]):
        cmd = ["g++", "-O2", "-std=c++17", f"-I{INCLUDE}", "-o", exe] + srcs + \
              [f"-L{PKG}", "-lbsfh", f"-Wl,-rpath,{PKG}", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host build failed: {' '.join(cmd)}\n{r.stderr}")
    return exe


def build_all(force=False):
    lib = build_library(force=force)
    exe = build_host(force=force)
    return lib, exe


if __name__ == "__main__":
    print(build_all(force=True))
