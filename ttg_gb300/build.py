"""Build recipe for the sm_103a shared library (libgbx_potrf.so), in-tree.

Every .cu under csrc/ is compiled with nvcc for sm_103a only (one -gencode), in parallel, and
linked into one shared library with a C ABI (include/gbx_potrf.h). No cmake, no torch
extension machinery: the library has no torch types in its interface.
"""
import concurrent.futures as cf
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbx_potrf.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-DGBX_ARCH=1030",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")))
    objs, jobs = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if verbose and (r.stdout or r.stderr):
                    print(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed: %s\n%s%s" % (" ".join(j), r.stdout, r.stderr))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(LIB + ".tmp", LIB)
    return LIB


DRIVER_SRC = os.path.join(HERE, "potrf", "testing_dpotrf.cc")
DRIVER = os.path.join(HERE, "potrf", "testing_dpotrf")


def build_driver(force=False):
    """The potrf flowgraph driver on the TTG API (C++ host code linked to libgbx_potrf.so)."""
    lib = build()
    deps = [DRIVER_SRC, lib, os.path.join(HERE, "potrf", "potrf.h"), os.path.join(HERE, "potrf", "potrs.h"),
            os.path.join(HERE, "potrf", "matrix.h")]
    deps += glob.glob(os.path.join(INCLUDE, "ttg", "*.h")) + glob.glob(os.path.join(INCLUDE, "ttg", "*", "*.h"))
    if force or _stale(DRIVER, deps):
        cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))) if os.path.isabs(nvcc()) else "/usr/local/cuda"
        cmd = ["g++", "-std=c++20", "-O2", "-pthread", "-I", INCLUDE, "-I", os.path.join(HERE, "potrf"),
               "-I", os.path.join(cuda, "include"), DRIVER_SRC, "-o", DRIVER, "-L", HERE, "-lgbx_potrf",
               "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + HERE]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("driver build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return DRIVER


CHAIN_SRC = os.path.join(HERE, "potrf", "chain_dev.cc")
CHAIN = os.path.join(HERE, "potrf", "chain_dev")


def build_chain(force=False):
    """The device-task chain benchmark on the TTG API (per-task runtime overhead)."""
    lib = build()
    deps = [CHAIN_SRC, lib] + glob.glob(os.path.join(INCLUDE, "ttg", "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "ttg", "*", "*.h"))
    if force or _stale(CHAIN, deps):
        cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))) if os.path.isabs(nvcc()) else "/usr/local/cuda"
        cmd = ["g++", "-std=c++20", "-O2", "-pthread", "-I", INCLUDE, "-I", os.path.join(cuda, "include"), CHAIN_SRC,
               "-o", CHAIN, "-L", HERE, "-lgbx_potrf", "-L", os.path.join(cuda, "lib64"), "-lcudart",
               "-Wl,-rpath," + HERE]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("chain benchmark build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return CHAIN


if __name__ == "__main__":
    print(build(force=True, verbose=True))
    print(build_driver(force=True))
    print(build_chain(force=True))
