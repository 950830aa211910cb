"""Build the in-tree shared library libswpc_gb300.so for sm_103a.

The library holds the CUDA kernels, the C ABI of include/swpc_gpu.h and the
host driver layer.  Translation units are compiled in parallel with nvcc and
linked with nvcc; the result lands in openswpc_gb300/_build/.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libswpc_gb300.so")
DRIVER = os.path.join(BUILD, "swpc_3d_gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off"]

CU_SOURCES = ["swpc_gpu.cu"]
CXX_SOURCES = ["host.cpp", "serve.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".hpp", ".cpp", ".h"))]
    files.append(os.path.join(ROOT, "include", "swpc_gpu.h"))
    return files


def _stale(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(force=False, verbose=False):
    """Compile every translation unit for sm_103a and link the shared library
    and the command-line driver.  Returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and not _stale(LIB) and not _stale(DRIVER):
        return LIB
    nvcc = _nvcc()
    jobs = []
    objs = []
    for f in CU_SOURCES:
        o = os.path.join(BUILD, f + ".o")
        objs.append(o)
        jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, f), "-o", o])
    for f in CXX_SOURCES:
        o = os.path.join(BUILD, f + ".o")
        objs.append(o)
        jobs.append(["g++", *CXX_FLAGS, "-I/usr/local/cuda/include", "-c", os.path.join(CSRC, f), "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
        return r.stdout

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"])
    os.replace(tmp, LIB)
    drv_src = os.path.join(CSRC, "driver_main.cpp")
    if os.path.exists(drv_src):
        run(["g++", *CXX_FLAGS, "-o", DRIVER + ".tmp", drv_src, "-L" + BUILD, "-lswpc_gb300",
             "-Wl,-rpath,$ORIGIN"])
        os.replace(DRIVER + ".tmp", DRIVER)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
