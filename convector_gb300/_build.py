"""In-tree build of libconvector_gpu.so for sm_103a.

Host C++ (OBJ loader, BVH build) is compiled with g++ and -ffp-contract=off;
the CUDA sources with nvcc for sm_103a only and -fmad=false, so that every
floating-point operation rounds where the reference's AVX code rounds.
Translation units compile in parallel; the link is skipped when the library
is newer than every source.
"""

import concurrent.futures
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib", "libconvector_gpu.so")
# The L2 read-bandwidth probe (the traversal kernels' L2 roofline), a library
# of its own: the render path never loads it.
PROBE_SOURCE = "l2_probe.cu"
PROBE_LIB = os.path.join(PKG, "lib", "libconvector_l2probe.so")

CU_SOURCES = ["kernels.cu", "wavefront.cu", "engine.cu", "capi.cu", "noalloc.cu", "postprocess.cu", "bvh_build.cu"]
CPP_SOURCES = ["host_scene.cpp"]
HEADERS = ["x86sem.cuh", "layout.cuh", "traverse.cuh", "shade.cuh", "path_refill.cuh", "kernels.h", "internal.h",
           "x86_approx_tables.h", "wavefront.cuh", "engine.h", "device_guard.cuh"]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-lineinfo", "-O3", "-std=c++17",
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build convector_gb300")


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def _run(cmd):
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), res.stdout))
    return res.stdout


def build_probe(force=False):
    """Compiles libconvector_l2probe.so if its source is newer; returns its path."""
    src = os.path.join(CSRC, PROBE_SOURCE)
    if not force and os.path.exists(PROBE_LIB) and os.path.getmtime(PROBE_LIB) >= _newest([src, __file__]):
        return PROBE_LIB
    os.makedirs(os.path.dirname(PROBE_LIB), exist_ok=True)
    tmp = "%s.%d.tmp" % (PROBE_LIB, os.getpid())  # concurrent builds must not share it
    _run([_nvcc()] + NVCC_FLAGS + ["-shared", "-o", tmp, src])
    os.replace(tmp, PROBE_LIB)
    return PROBE_LIB


def build(force=False, verbose=False, extra_nvcc=()):
    """Compiles the extension if any source is newer than the library; returns its path."""
    sources = [os.path.join(CSRC, s) for s in CU_SOURCES + CPP_SOURCES + HEADERS]
    sources.append(os.path.join(INCLUDE, "convector_gpu.h"))
    sources.append(os.path.abspath(__file__))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest(sources) and not extra_nvcc:
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    nvcc = _nvcc()
    cxx = os.environ.get("CXX", "g++")
    jobs = []
    objs = []
    for s in CU_SOURCES:
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        jobs.append([nvcc] + NVCC_FLAGS + list(extra_nvcc) + ["-I", INCLUDE, "-c", os.path.join(CSRC, s), "-o", obj])
    for s in CPP_SOURCES:
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        jobs.append([cxx] + CXX_FLAGS + ["-I", INCLUDE, "-c", os.path.join(CSRC, s), "-o", obj])
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs) + 1) as ex:
        probe = ex.submit(build_probe, force)
        outs = list(ex.map(_run, jobs))
        probe.result()
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = "%s.%d.tmp" % (LIB, os.getpid())
    _run([nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs
         + ["-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
