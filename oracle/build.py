"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/libfim_oracle.so`` -- the C restatement in fim_oracle.c.
* ``oracle/_ref/libfimref.so`` -- the reference's own host-compilable code
  (local solver, preprocessing, VTK/JSON I/O) compiled from the reference
  sources where they lie, plus ref_shim.cpp.  Built only when the reference
  tree is present (it is not shipped with this repository).

Usage: ``python oracle/build.py [--ref-root DIR]`` (default: $FIM_REFERENCE_ROOT,
else ``../reference`` beside the repository).
"""
import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CUDA_INC = "/usr/local/cuda/include"


def reference_root():
    """Checkout of the reference: $FIM_REFERENCE_ROOT, else a ``reference``
    directory beside this repository."""
    env = os.environ.get("FIM_REFERENCE_ROOT")
    if env:
        return env
    return os.path.normpath(os.path.join(HERE, "..", "..", "reference"))


DEFAULT_REF = reference_root()


def build_oracle(verbose=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libfim_oracle.so")
    src = os.path.join(HERE, "fim_oracle.c")
    if os.path.exists(out) and os.path.getmtime(out) > os.path.getmtime(src):
        return out
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           src, "-o", out, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return out


def build_ref(ref_root=DEFAULT_REF, verbose=False):
    """Compile the reference's host code into oracle/_ref/libfimref.so."""
    if not os.path.isdir(os.path.join(ref_root, "src", "eikonal")):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libfimref.so")
    shim = os.path.join(HERE, "ref_shim.cpp")
    srcs = [os.path.join(ref_root, "src", p) for p in (
        "core/types.cpp", "core/logging.cpp", "core/excepts.cpp", "core/sorts.cpp",
        "io/vtk.cpp", "io/io_json.cpp", "io/io_base.cpp")]
    newest = max(os.path.getmtime(p) for p in srcs + [shim])
    if os.path.exists(out) and os.path.getmtime(out) > newest:
        return out
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-I" + ref_root, "-I" + os.path.join(ref_root, "src"), "-I" + CUDA_INC,
           shim] + srcs + ["-o", out]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return out


def build_ref_driver(ref_root=DEFAULT_REF, verbose=False):
    """Compile oracle/ref_types_driver.cpp against the reference's real types
    and readers (its sources where they lie) and this repository's drop-in
    solver class and library into oracle/_ref/ref_types_driver.  Returns the
    path, or None without the reference tree or the built library."""
    if not os.path.isdir(os.path.join(ref_root, "src", "eikonal")):
        return None
    repo = os.path.dirname(HERE)
    lib_dir = os.path.join(repo, "cufim-nvlink_gb300", "_build")
    if not os.path.exists(os.path.join(lib_dir, "libfim_gb300.so")):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "ref_types_driver")
    drv = os.path.join(HERE, "ref_types_driver.cpp")
    shim = os.path.join(repo, "cufim-nvlink_gb300", "csrc", "cuda_solver_fim.cpp")
    srcs = [os.path.join(ref_root, "src", p) for p in (
        "core/types.cpp", "core/logging.cpp", "core/excepts.cpp", "core/sorts.cpp",
        "io/vtk.cpp", "io/io_json.cpp", "io/io_base.cpp")]
    deps = srcs + [drv, shim, os.path.join(repo, "cufim-nvlink_gb300", "csrc", "cuda_solver_fim.h"),
                   os.path.join(lib_dir, "libfim_gb300.so")]
    if os.path.exists(out) and os.path.getmtime(out) > max(os.path.getmtime(p) for p in deps):
        return out
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-fopenmp", "-I" + ref_root, "-I" + os.path.join(ref_root, "src"),
           "-I" + repo, "-I" + CUDA_INC, drv, shim] + srcs + [
           "-L" + lib_dir, "-lfim_gb300", "-Wl,-rpath," + lib_dir, "-o", out]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=DEFAULT_REF)
    a = ap.parse_args()
    print(build_oracle(verbose=True))
    print(build_ref(a.ref_root, verbose=True))
    print(build_ref_driver(a.ref_root, verbose=True))
