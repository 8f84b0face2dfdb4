"""Build of the native parts: libgbp.so (CUDA, sm_103a) and the SCIP propagator plugin core.

nvcc is called directly (no torch extension machinery): the product is a plain C-ABI shared library.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIBGBP = os.path.join(LIBDIR, "libgbp.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "--fmad=false", "-std=c++17",
              "-Xcompiler", "-fPIC", "-I" + INCLUDE]
CU_SOURCES = ["gbp_kernels.cu", "gbp_nodes_ranged.cu", "gbp_api.cu", "gbp_noalloc.cu", "gbp_seq.cu", "gbp_server.cu"]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build_libgbp(force: bool = False, verbose: bool = False) -> str:
    """Compile the CUDA sources (one object each, in parallel) and link libgbp.so."""
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "gbp.h"))
    srcs = [os.path.join(CSRC, f) for f in CU_SOURCES]
    if not force and _newer(LIBGBP, srcs + headers):
        return LIBGBP
    nvcc = _nvcc()
    objs = [os.path.join(LIBDIR, os.path.basename(s) + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        cmd = [nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", LIBGBP] + objs + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIBGBP


if __name__ == "__main__":
    print(build_libgbp(force=True, verbose=True))
