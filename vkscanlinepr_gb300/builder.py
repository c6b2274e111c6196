"""Builds libsr.so (the CUDA scanline renderer) in-tree for sm_103a.

Each .cu translation unit compiles in parallel with one -gencode; device code
uses --fmad=false and IEEE division/square root, host code -ffp-contract=off,
so no multiply-add is ever fused on either side.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsr.so")
REPO = os.path.dirname(HERE)

CU_SOURCES = ["geom.cu", "scan.cu", "sort.cu", "winding.cu", "resolve.cu", "mlp.cu", "segsort.cu", "api.cu", "noalloc.cu"]
CPP_SOURCES = ["host.cpp", "server.cpp", "image.cpp"]
HEADERS = ["common.cuh", "kernels.h", "synth.h"]

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(c):
            return c
    return "/usr/local/cuda"


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(REPO, "include", "sr.h")]
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            jobs.append([NVCC] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj])
    inc = os.path.join(_cuda_home(), "include")
    for s in CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-I", inc, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        return cmd, r.returncode, r.stdout

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, rc, out in ex.map(run, jobs):
                log = os.path.join(BUILD, os.path.basename(cmd[-1]) + ".log")
                with open(log, "w") as f:
                    f.write(" ".join(cmd) + "\n" + out)
                if rc != 0:
                    sys.stderr.write(out)
                    raise RuntimeError("compile failed: " + " ".join(cmd))
                if verbose:
                    sys.stdout.write(out)
    if force or jobs or _newer(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-ldl", "-lrt", "-lpthread"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
