"""Build recipe of the CUDA library (sm_103a) and its host-side math shim.

``python -m pixels_gb300.build`` compiles, in parallel, the kernels and the
host runtime with nvcc and links ``pixels_gb300/libpixels_gb300.so`` in-tree.
Device code is compiled with ``-fmad=false`` and host code with
``-ffp-contract=off``: the float64 path must round every operation like a
JavaScript number.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libpixels_gb300.so")
JSM_OUT = os.path.join(HERE, "libpx_jsmath_host.so")
BUILD_DIR = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-fmad=false", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-Xptxas", "-warn-spills"]
UNITS = ["kernels.cu", "px_api.cu", "px_serve.cu", "px_noalloc.cu", "px_lights.cu"]
HEADERS = ["px_internal.cuh", "sdf64.cuh", "sdf32.cuh", "paint.cuh", "paint32.cuh", "jsmath.cuh", "jsmath_tables.h"]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, defines=(), out: str = OUT) -> str:
    """Compile and link the library; ``defines`` (``NAME=VALUE``) select kernel
    variants (register budgets) and ``out`` an alternative output path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    tag = "_".join(d.replace("=", "") for d in defines)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "pixels_gb300.h")]
    objs = []
    jobs = []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD_DIR, u.replace(".cu", f"{tag}.o"))
        objs.append(obj)
        if force or _stale(obj, [src, *hdrs, __file__]):
            jobs.append([_nvcc(), *ARCH, *NVCC_FLAGS, *[f"-D{d}" for d in defines], "-c", src, "-o", obj])
    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(out, objs):
        run([_nvcc(), *ARCH, "-shared", "-o", out, *objs, "-lcudart"])
    jsrc = os.path.join(CSRC, "jsmath_host.cpp")
    if force or _stale(JSM_OUT, [jsrc, os.path.join(CSRC, "jsmath.cuh"), os.path.join(CSRC, "jsmath_tables.h")]):
        run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-o", JSM_OUT, jsrc])
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
