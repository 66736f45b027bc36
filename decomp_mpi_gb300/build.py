"""Build the in-tree shared library ``libdecomp_gb300.so``.

Host C sources are compiled with gcc, CUDA sources with nvcc for sm_103a
only, in parallel, and linked by nvcc with the static CUDA runtime.  The
library lands next to this file so that tests, ``bench.py`` and user code
load the in-tree build.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
INCLUDE_DIR = os.path.join(REPO_DIR, "include")
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libdecomp_gb300.so"
LIB_PATH = os.path.join(PKG_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
CC = os.environ.get("CC", "gcc")
# extra nvcc flags, e.g. "-DDMG_FFT_MINB=2" to try another register budget
NVCC_EXTRA = os.environ.get("DMG_NVCC_FLAGS", "").split()


def _sources():
    host = sorted(glob.glob(os.path.join(CSRC, "host", "*.c")))
    cuda = sorted(glob.glob(os.path.join(CSRC, "kernels", "*.cu")))
    return host, cuda


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _obj(src):
    base = os.path.relpath(src, CSRC).replace(os.sep, "_")
    return os.path.join(BUILD_DIR, base + ".o")


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile every source that changed and link the library; returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    host, cuda = _sources()
    headers = (glob.glob(os.path.join(INCLUDE_DIR, "*.h")) + glob.glob(os.path.join(CSRC, "*", "*.h")) +
               glob.glob(os.path.join(CSRC, "*", "*.cuh")))
    incs = ["-I" + INCLUDE_DIR, "-I" + os.path.join(CSRC, "host")]
    jobs = []
    for s in host:
        o = _obj(s)
        if force or _stale(o, [s] + headers):
            jobs.append([CC, "-O2", "-g", "-fPIC", "-std=gnu11", "-Wall", "-Wno-unused-function",
                         *incs, "-c", s, "-o", o])
    for s in cuda:
        o = _obj(s)
        if force or _stale(o, [s] + headers):
            jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "--expt-relaxed-constexpr", *NVCC_EXTRA, *incs, "-c", s, "-o", o])
    if jobs:
        # the pass kernels take longest: start them first, on every host core
        jobs.sort(key=lambda j: (j[0] != NVCC, -os.path.getsize(j[-3])))
        with ThreadPoolExecutor(max_workers=min(max(8, os.cpu_count() or 8), len(jobs))) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for j, o in zip(jobs, outs):
                print(" ".join(j))
                if o.strip():
                    print(o)
    objs = [_obj(s) for s in host + cuda]
    if force or jobs or _stale(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp"
        _run([NVCC, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread", "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
