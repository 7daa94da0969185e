"""Build the GB300 (sm_103a) library in-tree.

Compiles every CUDA source for sm_103a (``-gencode arch=compute_103a,code=sm_103a``),
the host C++ with g++, and links ``respackdev_gb300/lib/librespack_gb300.so`` plus
the ``respackdev_gb300/bin/rp_calc_chiqw``, ``rp_calc_w3d`` and ``rp_calc_j3d`` executables.  Objects go to
``respackdev_gb300/_build``.  Compilation runs in parallel; a file is rebuilt when
it or any header is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
BINDIR = os.path.join(HERE, "bin")
LIB = os.path.join(LIBDIR, "librespack_gb300.so")
EXE = os.path.join(BINDIR, "rp_calc_chiqw")
# executables: main source -> program (drop-ins for calc_chiqw, calc_w3d, calc_j3d)
MAINS = {"rp_main.cpp": "rp_calc_chiqw", "rp_main_w3d.cpp": "rp_calc_w3d", "rp_main_j3d.cpp": "rp_calc_j3d"}
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# files whose arithmetic should round like the CPU reference (no FMA contraction)
NOFMAD: set = set()
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function", f"-I{CUDA_HOME}/include"]


def _newest_header() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    return max(os.path.getmtime(h) for h in hs) if hs else 0.0


def _compile(src: str, obj: str, verbose: bool) -> str:
    name = os.path.basename(src)
    if src.endswith(".cu"):
        cmd = [NVCC] + ARCH + NVFLAGS + (["--fmad=false"] if name in NOFMAD else []) + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXXFLAGS + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {name}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    hdr = _newest_header()
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    lib_srcs = [s for s in srcs if os.path.basename(s) not in MAINS]
    jobs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr):
            jobs.append((s, o))
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        for msg in ex.map(lambda j: _compile(j[0], j[1], verbose), jobs):
            if msg and verbose:
                print(msg, file=sys.stderr)
    objs = [os.path.join(BUILD, os.path.basename(s) + ".o") for s in lib_srcs]
    newest = max(os.path.getmtime(o) for o in objs)
    if force or jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp"
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    for src, prog in MAINS.items():
        main_o = os.path.join(BUILD, src + ".o")
        exe = os.path.join(BINDIR, prog)
        if force or not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(LIB), os.path.getmtime(main_o)):
            cmd = ["g++", "-o", exe, main_o, f"-L{LIBDIR}", "-lrespack_gb300", "-Wl,-rpath,$ORIGIN/../lib",
                   f"-L{CUDA_HOME}/lib64", "-lcudart"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link of {prog} failed\n{r.stderr}")
    return LIB


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
