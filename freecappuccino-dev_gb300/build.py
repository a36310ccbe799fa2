"""Build recipe of libfcgpu.so: every CUDA translation unit for sm_103a plus the
C++ host runtime, compiled in parallel, linked into one shared library next to
this file.  Used by __graft_entry__.build() and the tests; no cmake.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfcgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + INCLUDE, "-I" + CSRC, "-I" + HOST]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off", "-I" + INCLUDE, "-I" + HOST, "-I" + CSRC]
# Translation units whose FP64 expressions are written in the reference's
# evaluation order and must not be contracted into FMAs.
PER_FILE = {"fc_simple.cu": ["--fmad=false"], "fc_adjoint.cu": ["--fmad=false"], "fc_limiter.cu": ["--fmad=false"],
            "fc_nodegrad.cu": ["--fmad=false"]}


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    cu = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp"))
    return cu, cpp


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = sources()
    headers = [os.path.join(INCLUDE, "fc_gpu.h")] + [os.path.join(CSRC, f) for f in os.listdir(CSRC)
                                                     if f.endswith((".hpp", ".cuh"))] + \
              [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".hpp")]
    cmds = []
    objs = []
    for s in cu:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            cmds.append([nvcc] + ARCH + NVCC_FLAGS + PER_FILE.get(os.path.basename(s), []) + ["-c", s, "-o", o])
    for s in cpp:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            cmds.append(["g++"] + CXX_FLAGS + ["-c", s, "-o", o])

    def run(c):
        r = subprocess.run(c, capture_output=True, text=True)
        return c, r

    jobs = jobs or min(16, max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(jobs) as ex:
        for c, r in ex.map(run, cmds):
            if verbose or r.returncode:
                sys.stdout.write(" ".join(c[-3:]) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("compile failed: " + c[-3])
    if cmds or not os.path.exists(LIB) or _stale(LIB, objs):
        link = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode:
            sys.stdout.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
