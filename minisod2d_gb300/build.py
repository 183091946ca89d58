"""Build recipe for libmsod.so (the CUDA kernels, host setup code and C ABI).

Every translation unit is compiled in parallel -- CUDA sources by nvcc for
sm_103a only, the host setup code by g++ -- and linked in-tree into
``minisod2d_gb300/libmsod.so``.  No cmake, no torch extension machinery: the
library is a plain C-ABI shared object that Fortran, C, C++ or ctypes can load.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmsod.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + INCLUDE, "-I" + CSRC]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", "-I" + INCLUDE, "-I" + CSRC]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "msod.h"))
    files.append(os.path.join(HERE, "driver", "msod_driver.cpp"))
    return files


def _compile(args):
    cmd, log = args
    r = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, r.returncode, r.stdout + r.stderr


def build(force=False, verbose=False, ptxas_verbose=False):
    """Compile libmsod.so if any source is newer than it.  Returns its path."""
    if not force and os.path.exists(LIB) and os.path.exists(os.path.join(HERE, "msod_driver")):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(f) <= t for f in _deps()):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    cu, cpp = sources()
    jobs, objs = [], []
    for f in cu:
        obj = os.path.join(BUILD, f + ".o")
        extra = ["-Xptxas", "-v"] if ptxas_verbose else []
        # Compile-time kernel variants (e.g. -DCONVEC_MINB=3), for measuring.
        extra += os.environ.get("MSOD_NVCC_DEFINES", "").split()
        jobs.append(([_nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, f), "-o", obj], f))
        objs.append(obj)
    for f in cpp:
        obj = os.path.join(BUILD, f + ".o")
        jobs.append((["g++", *CXX_FLAGS, "-c", os.path.join(CSRC, f), "-o", obj], f))
        objs.append(obj)
    workers = max(1, min(len(jobs), os.cpu_count() or 1))
    failed = []
    with ThreadPoolExecutor(workers) as ex:
        for cmd, rc, out in ex.map(_compile, jobs):
            if verbose or rc != 0 or ptxas_verbose:
                print(" ".join(cmd))
                if out:
                    print(out)
            if rc != 0:
                failed.append(cmd[-3])
    if failed:
        raise RuntimeError("libmsod build failed: " + ", ".join(failed))
    tmp = LIB + ".tmp"
    link = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        print(" ".join(link))
        print(r.stdout + r.stderr)
        raise RuntimeError("libmsod link failed")
    os.replace(tmp, LIB)
    build_driver()
    return LIB


DRIVER_SRC = os.path.join(HERE, "driver", "msod_driver.cpp")
DRIVER = os.path.join(HERE, "msod_driver")


def build_driver():
    """The benchmark driver executable (main.f90 on the C ABI), linked to libmsod.so."""
    tmp = DRIVER + ".tmp"
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I" + INCLUDE, "-I" + os.path.join(cuda, "include"), DRIVER_SRC,
           "-L" + HERE, "-lmsod", "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        print(" ".join(cmd))
        print(r.stdout + r.stderr)
        raise RuntimeError("msod_driver build failed")
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv))
