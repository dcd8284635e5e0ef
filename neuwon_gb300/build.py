"""Compile ``libneuwon_gb300.so`` for sm_103a with nvcc (in-tree, no cmake).

    python -m neuwon_gb300.build          # incremental
    python -m neuwon_gb300.build --force  # rebuild everything
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libneuwon_gb300.so")
SOURCES = ["nw_step_f32.cu", "nw_step_f64.cu", "nw_api.cu", "nw_step.cu", "nw_propagator.cu", "nw_noalloc.cu", "nw_adjoint.cu", "nw_tune.cu", "nw_wide.cu", "nw_species.cu", "nw_lti.cu"]
HEADERS = ["nw_internal.cuh", "nw_step_common.cuh", "nw_step_batched.cuh", os.path.join("..", "..", "include", "neuwon_gb300.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
         "--expt-relaxed-constexpr"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build neuwon_gb300")
    return path


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def build(force=False, verbose=False):
    """Build the shared library if any source or header is newer than it."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    hdrs = [os.path.normpath(os.path.join(CSRC, h)) for h in HEADERS]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest(srcs + hdrs):
        return LIB
    cc = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < _newest([src] + hdrs):
            cmd = [cc] + ARCH + FLAGS + ["-c", src, "-o", obj]
            if verbose:
                cmd += ["-Xptxas", "-v"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
            if verbose and r.stderr:
                print(r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
