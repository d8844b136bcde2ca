"""Builds the solver library and tools in-tree for sm_103a.

Outputs (under cufim-nvlink_gb300/_build/):
  * libfim_gb300.so -- the C ABI of include/fim.h (kernels + host staging + I/O)
  * fim_cli         -- the reference-compatible command line front end

The CUDA translation units are compiled with -fmad=false: the solver's FP64
arithmetic must follow the reference's source operation by operation.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
# FIM_BUILD_DIR + FIM_BUILD_DEFINES build a variant elsewhere (e.g.
# FIM_BUILD_DEFINES=FIM_PROBE for per-phase timing of the solve kernel)
if os.environ.get("FIM_BUILD_DIR"):
    OUT = os.environ["FIM_BUILD_DIR"]
DEFINES = ["-D" + x for x in os.environ.get("FIM_BUILD_DEFINES", "").split(",") if x]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["fim_kernels.cu", "fim_solve_s192.cu", "fim_solve_s160.cu", "fim_solve_s96.cu", "fim_static.cu",
              "fim_mlp.cu", "fim_selftest.cu"]
CPP_SOURCES = ["fim_solver.cpp", "fim_io.cpp", "cuda_solver_fim.cpp"]
CLI_SOURCES = ["fim_cli.cpp"]


def _needs(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    hs.append(os.path.join(HERE, "..", "include", "fim.h"))
    return hs


def _compile(src, verbose):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if not _needs(obj, [src] + _headers()):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC"] + DEFINES + [
               "-c", src, "-o", obj]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-I" + os.path.join(CUDA_HOME, "include")] + \
              DEFINES + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    return obj


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES + CPP_SOURCES + CLI_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    lib_objs = objs[:len(CU_SOURCES) + len(CPP_SOURCES)]
    cli_objs = objs[len(CU_SOURCES) + len(CPP_SOURCES):]
    lib = os.path.join(OUT, "libfim_gb300.so")
    cudalib = os.path.join(CUDA_HOME, "lib64")
    link_tail = ["-L" + cudalib, "-lcudart_static", "-lpthread", "-ldl", "-lrt", "-fopenmp"]
    if _needs(lib, lib_objs):
        cmd = ["g++", "-shared", "-o", lib] + lib_objs + link_tail
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    cli = os.path.join(OUT, "fim_cli")
    if _needs(cli, cli_objs + [lib]):
        cmd = ["g++", "-o", cli] + cli_objs + ["-L" + OUT, "-lfim_gb300", "-Wl,-rpath,$ORIGIN"] + link_tail
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
