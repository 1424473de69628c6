"""Build the engine's shared library in-tree for sm_103a.

    python -m kmc_dn_gb300.build   ->  kmc_dn_gb300/libkmc_dn_gb300.so

Each CUDA translation unit is compiled by its own nvcc process (in parallel)
with ``-gencode arch=compute_103a,code=sm_103a``, then linked into one
shared library exporting the C ABI of include/kmc_dn_gb300.h.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libkmc_dn_gb300.so")
# The same sources with -DKMC_DEBUG_CHECKS: the hop loop checks its decoded
# pair and list indices and stops a chain with KMC_ERR_INVALID instead of
# touching memory out of range (a stand-in for compute-sanitizer).
DEBUG_LIB = os.path.join(HERE, "libkmc_dn_gb300_debug.so")
# The same sources with -DKMC_SECTION_CLOCKS: the hop loop times its phases
# with the SM clock (kmc_section_clocks; kmc_dn_gb300/section_clocks.py).
CLOCKS_LIB = os.path.join(HERE, "libkmc_dn_gb300_clocks.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build kmc_dn_gb300")
    return exe


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale(lib=LIB):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = sources() + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    deps.append(os.path.join(os.path.dirname(HERE), "include", "kmc_dn_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(p) > t for p in deps)


def build(force=False, verbose=False, extra=(), debug_checks=False, section_clocks=False):
    if debug_checks and section_clocks:
        raise ValueError("build one of the debug-checks and section-clocks libraries at a time")
    lib = DEBUG_LIB if debug_checks else CLOCKS_LIB if section_clocks else LIB
    objdir = OBJ + ("_debug" if debug_checks else "_clocks" if section_clocks else "")
    if debug_checks:
        extra = tuple(extra) + ("-DKMC_DEBUG_CHECKS",)
    if section_clocks:
        extra = tuple(extra) + ("-DKMC_SECTION_CLOCKS",)
    if not force and not _stale(lib):
        return lib
    os.makedirs(objdir, exist_ok=True)
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        cmd = [exe, *ARCH, *FLAGS, *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stderr.strip() or r.stdout.strip()):
            print(r.stdout + r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(sources())) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = lib + f".tmp{os.getpid()}"
    cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = ("-Xptxas", "-v") if v else ()
    print(build(force=True, verbose=v, extra=extra, debug_checks="--debug-checks" in sys.argv,
                section_clocks="--section-clocks" in sys.argv))
