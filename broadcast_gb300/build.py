"""Build libbroadcast_gb300.so in-tree (broadcast_gb300/_lib/) for sm_103a.

Each CUDA translation unit is compiled by nvcc in parallel, the host
pre-processing unit by g++, and the objects are linked into one shared
library with the C ABI declared in include/broadcast_gb300.h.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libbroadcast_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CU_SOURCES = ["residual.cu", "bc.cu", "assembly.cu", "runtime.cu", "api.cu", "calib.cu", "noalloc.cu", "adjoint.cu", "jacobian.cu", "span.cu", "batch.cu", "schemes.cu", "impli.cu", "bandlu.cu", "krylov.cu", "mlp.cu"]
CPP_SOURCES = ["host.cpp"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbroadcast_gb300.so")
    return cand


def _cuda_root(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    """Compile the library if any source is newer than it; return its path."""
    nvcc = _nvcc()
    cuda = _cuda_root(nvcc)
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         "--expt-relaxed-constexpr", "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + os.path.join(cuda, "include"),
                         "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out:
                    sys.stdout.write(out)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-lcudart", "-lcublas", "-lcusolver"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
