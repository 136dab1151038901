"""Build ``lib/libgw_gb300.so`` (the C-ABI library) for sm_103a with nvcc.

Each translation unit is compiled in parallel, then linked into one shared
library with the CUDA runtime linked statically, so the library has no
dependency beyond the driver.  Host code is compiled with
``-ffp-contract=off``: the set-up classifies cells with float comparisons
that must round as the reference's scalar code does.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgw_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["gw_setup.cpp", "gw_setup_dev.cu", "gw_api.cu", "gw_kernels.cu", "gw_fused.cu", "gw_tridiag.cu",
           "gw_batch.cu", "gw_noalloc.cu", "gw_adjoint.cu"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


# The debug build (-DGW_DEBUG, lib/libgw_gb300_debug.so): the fused step's
# kernels check every global and shared-memory access (csrc/gw_debug.cuh) and
# report a failed check as GW_ERR_ARG instead of touching the address.
DEBUG_LIB = os.path.join(OUT_DIR, "libgw_gb300_debug.so")
DEBUG_OBJ_DIR = os.path.join(HERE, "_build_debug")


def _compile(src, verbose, debug=False):
    obj = os.path.join(DEBUG_OBJ_DIR if debug else OBJ_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
           "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj]
    if debug:
        cmd.insert(1, "-DGW_DEBUG")
    if src.endswith(".cpp"):
        cmd[cmd.index("-c"):cmd.index("-c")] = ["-x", "cu"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj, r.stdout + r.stderr


def _stale(lib=LIB):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "gw_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False, debug=False):
    """Compile the library (debug=True: the bounds-checking debug build) if
    any source is newer than it; returns its path."""
    lib = DEBUG_LIB if debug else LIB
    if not force and not _stale(lib):
        return lib
    os.makedirs(DEBUG_OBJ_DIR if debug else OBJ_DIR, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, debug), SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp] + [o for o, _ in results]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, debug="--debug" in sys.argv))
