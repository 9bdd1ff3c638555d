"""Native build of the package: the CUDA library (sm_103a), the synthetic-data
generator and the `tuna` CLI. Everything is built in-tree under
tuna_gb300/_build/ with nvcc/gcc directly (no CMake), compiled in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

GPU_LIB = os.path.join(BUILD, "libtuna_gpu.so")
SYNTH_LIB = os.path.join(BUILD, "libtuna_synth.so")
CLI_BIN = os.path.join(BUILD, "tuna")

# translation units of libtuna_gpu.so
CU_SOURCES = ["tg_api.cu", "tg_phase1.cu", "tg_phase2.cu", "tg_noalloc.cu", "tg_lex.cu", "tg_format.cu",
              "tg_link.cu", "tg_spill.cu"]
CPP_SOURCES = ["host/fastx.cpp", "host/output.cpp", "host/hostmem.cpp"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers():
    out = []
    for base in (CSRC, INCLUDE):
        for dp, _, fs in os.walk(base):
            out += [os.path.join(dp, f) for f in fs if f.endswith((".h", ".cuh", ".hpp"))]
    return out


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def synth_lib(build_if_missing: bool = True) -> str:
    src = os.path.join(CSRC, "synth.c")
    if build_if_missing and _newer(SYNTH_LIB, [src]):
        os.makedirs(BUILD, exist_ok=True)
        _run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-shared", "-fPIC", "-pthread",
              src, "-o", SYNTH_LIB + ".tmp"])
        os.replace(SYNTH_LIB + ".tmp", SYNTH_LIB)
    return SYNTH_LIB


def gpu_lib(build_if_missing: bool = True, verbose: bool = False) -> str:
    """Compile libtuna_gpu.so: .cu units for sm_103a plus the host C++ units."""
    if not build_if_missing:
        return GPU_LIB
    hdrs = _headers()
    objs = []
    jobs = []
    os.makedirs(os.path.join(BUILD, "obj"), exist_ok=True)
    nvcc = _nvcc()
    common_inc = ["-I", CSRC, "-I", INCLUDE]
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, "obj", os.path.basename(s) + ".o")
        objs.append(obj)
        if _newer(obj, [src] + hdrs):
            jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "--expt-relaxed-constexpr", "-Xptxas", "-v" if verbose else "-O3",
                         *common_inc, "-c", src, "-o", obj])
    for s in CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, "obj", os.path.basename(s) + ".o")
        objs.append(obj)
        if _newer(obj, [src] + hdrs):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-Wall", *common_inc,
                         "-I", "/usr/local/cuda/include", "-c", src, "-o", obj])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                sys.stdout.write(o)
    if jobs or not os.path.exists(GPU_LIB):
        _run([nvcc, *ARCH, "-shared", "-o", GPU_LIB + ".tmp", *objs, "-lcudart", "-lpthread", "-ldl"])
        os.replace(GPU_LIB + ".tmp", GPU_LIB)
    return GPU_LIB


def cli(build_if_missing: bool = True) -> str:
    """The drop-in `tuna` executable, linked against libtuna_gpu.so."""
    src = os.path.join(CSRC, "cli", "tuna_main.cpp")
    if build_if_missing and _newer(CLI_BIN, [src, GPU_LIB] + _headers()):
        _run(["g++", "-O2", "-std=c++20", "-Wall", "-I", INCLUDE, src, "-o", CLI_BIN + ".tmp",
              "-L", BUILD, "-ltuna_gpu", "-Wl,-rpath,$ORIGIN", "-lpthread"])
        os.replace(CLI_BIN + ".tmp", CLI_BIN)
    return CLI_BIN


def build_all(verbose: bool = False) -> None:
    synth_lib()
    gpu_lib(verbose=verbose)
    cli()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
