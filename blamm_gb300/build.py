"""Builds the native parts of blamm_gb300 in-tree (the test infrastructure -- the CPU oracle
and the reference binary -- has its own build, oracle/oracle_build.py).

  libblamm_gpu.so   CUDA kernels + the C ABI of include/blamm_gpu.h (sm_103a only)
  libblamm_host.so  C++ host library of include/blamm_host.h (motifs, PWMs,
                    histograms, FASTA streaming, occurrence output)
  bin/blamm         the drop-in `blamm dict|hist|scan` command line

Everything lands in blamm_gb300/_build (and blamm_gb300/bin); nothing is
installed.  Compilation units build in parallel.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
BIN = os.path.join(PKG, "bin")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
            "-Wno-unused-parameter"]
HOST_SRCS = ["motif.cpp", "sequence.cpp", "species.cpp", "histogram.cpp",
             "scan.cpp", "host_capi.cpp", "serve.cpp", "format.cpp", "ingest.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + res.stdout)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _gpu_lib(force: bool) -> str:
    out = os.path.join(BUILD, "libblamm_gpu.so")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh"))]
    deps.append(os.path.join(INCLUDE, "blamm_gpu.h"))
    if force or _stale(out, deps):
        _run([_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-shared", "-o", out,
              os.path.join(CSRC, "blamm_gpu.cu"), "-lcudart", "-ldl"])  # -ldl: NVTX finds its tool by dlopen
    return out


def _host_obj(src: str, force: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, "host", src)] + [
        os.path.join(CSRC, "host", h) for h in os.listdir(os.path.join(CSRC, "host"))
        if h.endswith(".h")] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    if force or _stale(obj, deps):
        _run(["g++", *CXXFLAGS, "-I", INCLUDE, "-c", os.path.join(CSRC, "host", src), "-o", obj])
    return obj


def _host(force: bool, pool: ThreadPoolExecutor) -> tuple[str, str]:
    objs = list(pool.map(lambda s: _host_obj(s, force), HOST_SRCS))
    lib = os.path.join(BUILD, "libblamm_host.so")
    if force or _stale(lib, objs):
        _run(["g++", "-shared", "-o", lib, *objs, "-L", BUILD, "-lblamm_gpu",
              "-Wl,-rpath,$ORIGIN", "-lpthread"])
    main_obj = _host_obj("blamm_main.cpp", force)
    exe = os.path.join(BIN, "blamm")
    gpu = os.path.join(BUILD, "libblamm_gpu.so")
    if force or _stale(exe, objs + [main_obj, gpu]):
        os.makedirs(BIN, exist_ok=True)
        _run(["g++", "-o", exe, main_obj, *objs, "-L", BUILD, "-lblamm_gpu",
              "-Wl,-rpath,$ORIGIN/../_build", "-lpthread"])
    return lib, exe


def build(force: bool = False) -> None:
    """Compile every native part of the product (GPU library, host library, CLI)."""
    os.makedirs(BUILD, exist_ok=True)
    # objects of another architecture (a copy built on x86 arriving on an Arm machine) are rebuilt
    stamp = os.path.join(BUILD, ".arch")
    arch = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch:
        force = True
    with ThreadPoolExecutor(max_workers=8) as pool:
        _gpu_lib(force)  # the CLI links the GPU library
        if all(os.path.exists(os.path.join(CSRC, "host", s)) for s in HOST_SRCS + ["blamm_main.cpp"]):
            _host(force, pool)
    with open(stamp, "w") as f:
        f.write(arch + "\n")


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("built:", BUILD)
