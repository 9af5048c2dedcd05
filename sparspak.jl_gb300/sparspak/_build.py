"""Build the two native libraries of the package, in-tree.

* ``_lib/libspk_host.so`` - host structure phase (graph, orderings,
  elimination tree, symbolic factorisation), C++17.
* ``_lib/libspk_gpu.so``  - the sm_103a numeric engine behind the C ABI of
  ``include/spk_gpu.h``, CUDA C++.

Both compile in parallel; a library is rebuilt only when a source is newer.
"""
from __future__ import annotations

import os
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                      # sparspak.jl_gb300/
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
LIBDIR = os.path.join(PKG, "_lib")

HOST_SO = os.path.join(LIBDIR, "libspk_host.so")
GPU_SO = os.path.join(LIBDIR, "libspk_gpu.so")

HOST_SRC = [os.path.join(CSRC, "spk_symbolic.cpp")]
GPU_SRC = [os.path.join(CSRC, "spk_gpu.cu"), os.path.join(CSRC, "spk_probe.cu")]
GPU_DEPS = GPU_SRC + [os.path.join(CSRC, "spk_kernels.cuh"), os.path.join(CSRC, "spk_umma.cuh"),
                      os.path.join(INCLUDE, "spk_gpu.h")]
HOST_DEPS = HOST_SRC + [os.path.join(INCLUDE, "spk_host.h")]

NVCC = os.environ.get("SPK_NVCC", "nvcc")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def host_cmd() -> list[str]:
    return ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
            "-o", HOST_SO] + HOST_SRC


def gpu_cmd() -> list[str]:
    return [NVCC, ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
            "-shared", "-o", GPU_SO] + GPU_SRC


def build(force: bool = False, verbose: bool = False) -> None:
    """Compile whatever is missing or out of date; raise on failure."""
    os.makedirs(LIBDIR, exist_ok=True)
    jobs = []
    if force or _stale(HOST_SO, HOST_DEPS):
        jobs.append(("libspk_host.so", host_cmd()))
    if force or _stale(GPU_SO, GPU_DEPS):
        jobs.append(("libspk_gpu.so", gpu_cmd()))
    procs = []
    for name, cmd in jobs:
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((name, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for name, cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"building {name} failed ({' '.join(cmd)}):\n{out.decode(errors='replace')}")
        elif verbose and out:
            print(out.decode(errors="replace"))
    if errors:
        raise RuntimeError("\n".join(errors))


if __name__ == "__main__":
    build(force=True, verbose=True)
