"""Builds the miner's native library and CLI in-tree.

Outputs (git-ignored): gpu_graph_mining_gb300/_lib/libgspan_gb300.so and
gpu_graph_mining_gb300/_lib/gspan_gb300.  CUDA code is compiled for sm_103a
only; host C++ with g++.  Translation units compile in parallel.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libgspan_gb300.so")
CLI = os.path.join(OUT, "gspan_gb300")
CONVERT = os.path.join(OUT, "gspan_gb300_convertdb")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SRCS = ["gs_kernels.cu", "gs_wave.cu", "gs_ismin.cu", "gs_ingest.cu", "gs_noalloc.cu"]
CPP_SRCS = ["gs_db.cpp", "gs_dfs.cpp", "gs_engine.cpp", "gs_capi.cpp", "gs_server.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "gspan_gb300.h"))
    jobs = []
    objs = []
    for s in CU_SRCS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s + ".o")
        objs.append(obj)
        if force or not _newer(obj, [src] + headers):
            jobs.append([NVCC] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                                         "-c", src, "-o", obj])
    for s in CPP_SRCS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s + ".o")
        objs.append(obj)
        if force or not _newer(obj, [src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-Wall",
                         "-I" + os.path.join(CUDA_HOME, "include"), "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                sys.stdout.write(out)
    if force or jobs or not os.path.exists(LIB):
        _run([NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs +
             ["-Xlinker", "--exclude-libs,ALL", "-lpthread"])
    for src, exe in ((os.path.join(CSRC, "gs_cli.cpp"), CLI), (os.path.join(CSRC, "gs_convertdb.cpp"), CONVERT)):
        if force or not _newer(exe, [src, LIB]):
            _run(["g++", "-O2", "-std=c++17", src, "-o", exe, "-L" + OUT, "-lgspan_gb300", "-Wl,-rpath,$ORIGIN"])
    return LIB


def clean():
    shutil.rmtree(OUT, ignore_errors=True)


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print(LIB)
