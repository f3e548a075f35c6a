"""In-tree build of libltpmg_gb300.so (sm_103a) with nvcc and g++.

Translation units compile in parallel into ltpmg_gb300/_build/ and link into
ltpmg_gb300/libltpmg_gb300.so.  No cmake, one -gencode, a minute or less.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libltpmg_gb300.so")
DEBUG_LIB = os.path.join(PKG, "libltpmg_gb300_debug.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(ROOT, "include")]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", os.path.join(ROOT, "include")]

CU_SOURCES = ["ltp_kernels.cu", "ltp_api.cu", "ltp_noalloc.cu", "ltp_ingest.cu"]
# the benchmark's random-access probe: its own library, outside the product
PROBE_SOURCE = "ltp_probe.cu"
PROBE_LIB = os.path.join(PKG, "libltpmg_probe.so")
CXX_SOURCES = ["ltp_gen.cpp", "ltp_compat.cpp", "ltp_serve.cpp", "ltp_tpcc.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose=False, extra_nvcc=(), debug_bounds=False):
    """debug_bounds: build libltpmg_gb300_debug.so with every scatter index
    checked against its capacity (-DLTP_DEBUG_BOUNDS) instead of the
    release library."""
    build_dir, lib = (BUILD + "_debug", DEBUG_LIB) if debug_bounds else (BUILD, LIB)
    if debug_bounds:
        extra_nvcc = tuple(extra_nvcc) + ("-DLTP_DEBUG_BOUNDS",)
    os.makedirs(build_dir, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = os.path.join(build_dir, src + ".o")
        objs.append(obj)
        jobs.append([nvcc] + ARCH + NVCC_FLAGS + list(extra_nvcc) + ["-c", os.path.join(CSRC, src), "-o", obj])
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")  # NVTX headers
    for src in CXX_SOURCES:
        obj = os.path.join(build_dir, src + ".o")
        objs.append(obj)
        jobs.append(["g++"] + CXX_FLAGS + ["-I", cuda_inc, "-c", os.path.join(CSRC, src), "-o", obj])
    probe_job = None
    if not debug_bounds:
        probe_job = [nvcc] + ARCH + NVCC_FLAGS + ["-shared", os.path.join(CSRC, PROBE_SOURCE), "-o", PROBE_LIB + ".tmp"]
        jobs.append(probe_job)
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if probe_job:
        os.replace(PROBE_LIB + ".tmp", PROBE_LIB)
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = lib + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
