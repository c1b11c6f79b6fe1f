"""Builds libsi_cuda.so in-tree (shaderintel_gb300/_build/) for sm_103a with nvcc and g++.

The kernels are compiled with -fmad=false: their f32 evaluation order (every operation rounded on
its own) is what makes the grid sums and particle state bit-identical to the CPU oracle. Host code
is compiled with -ffp-contract=off for the same reason (it restates the reference's f64 JavaScript
arithmetic). Translation units compile in parallel; one -gencode keeps the build to a minute.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsi_cuda.so")
INCLUDE = os.path.join(ROOT, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["si_kernels.cu", "si_sort.cu", "si_couple.cu", "si_emit.cu"]
CPP_SOURCES = ["si_runtime.cpp", "si_host.cpp", "si_server.cpp"]


def _sources():
    return [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES] + [
        os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))
    ] + [os.path.join(INCLUDE, "si_cuda.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _sources())


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(force=False, verbose=False, out_dir=None, defines=()):
    """Compile the CUDA library (if its sources changed) and return its path. out_dir/defines make
    a variant build (e.g. -DSI_G2P_MIN_CTAS=3) beside the default one."""
    global OUT, LIB
    if out_dir is not None:
        saved = (OUT, LIB)
        OUT, LIB = out_dir, os.path.join(out_dir, "libsi_cuda.so")
        try:
            return build(force, verbose, None, defines)
        finally:
            OUT, LIB = saved
    if not force and not _stale():
        return LIB
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(OUT, exist_ok=True)
    inc = ["-I" + CSRC, "-I" + INCLUDE, "-I" + os.path.join(CUDA_HOME, "include")]
    jobs = []
    for f in CU_SOURCES:
        obj = os.path.join(OUT, f + ".o")
        jobs.append(([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true",
                                      "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                                      "-c", os.path.join(CSRC, f), "-o", obj] + list(defines) + inc, obj))
    cxx = os.environ.get("CXX", "g++")
    for f in CPP_SOURCES:
        obj = os.path.join(OUT, f + ".o")
        jobs.append(([cxx, "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-c",
                      os.path.join(CSRC, f), "-o", obj] + inc, obj))
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-o", tmp] + [j[1] for j in jobs] + ["-lpthread"])
    os.replace(tmp, LIB)
    return LIB


def build_oracle():
    """Compile the CPU oracle (test infrastructure) with its Makefile."""
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    return os.path.join(ROOT, "oracle", "_build", "libsi_oracle.so")


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
    print(build_oracle())
