"""In-tree build of libcsem_gpu.so (CUDA kernels for sm_103a + the host C layer) and of
the key=value driver `csem`. Outputs go to demo_matrixfree_csem_gb300/_build/.

  python -m demo_matrixfree_csem_gb300.build [--force] [--verbose]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
# CSEM_BUILD_DIR puts a build elsewhere (e.g. variants built with CSEM_NVCC_FLAGS)
OUT = os.environ.get("CSEM_BUILD_DIR") or os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libcsem_gpu.so")
DRIVER = os.path.join(OUT, "csem")
REFABI = os.path.join(OUT, "libcsem_refabi.so")
# the host set-up alone (model read, padding, airwave tables; no CUDA), for CPU-only users
HOST_LIB = os.path.join(OUT, "libcsem_host.so")
INCLUDE = os.path.join(ROOT, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["k_fdfd.cu", "k_airwave.cu", "k_lusgs.cu", "k_lusgs2.cu", "k_lusgs3.cu", "k_lusgs4.cu", "k_lusgs5.cu", "k_blas.cu", "k_scalar.cu", "k_acq.cu",
              "engine_model.cu", "solve_fp64.cu", "solve_mixed.cu", "prof.cu", "capi.cu", "capi_noalloc.cu",
              "csr_compare.cu"]
C_SOURCES = ["csem_getpar.c", "csem_setup.c", "csem_partition.c"]
DRIVER_SOURCES = ["csem_main.c"]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout, r.stderr, flush=True)


def _compile_cu(src: str, obj: str, verbose: bool, extra: list[str]) -> str:
    cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I", INCLUDE, "-c", src, "-o", obj, *extra, *os.environ.get("CSEM_NVCC_FLAGS", "").split()]
    _run(cmd, verbose)
    return obj


def _compile_c(src: str, obj: str, verbose: bool) -> str:
    cmd = ["gcc", "-O3", "-fPIC", "-ffp-contract=off", "-std=gnu99", "-Wall", "-I", INCLUDE, "-c", src,
           "-o", obj]
    _run(cmd, verbose)
    return obj


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile every translation unit for sm_103a and link libcsem_gpu.so + csem."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(OUT, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        for s in CU_SOURCES:
            src, obj = os.path.join(CSRC, s), os.path.join(OUT, s + ".o")
            objs.append(obj)
            if force or ptxas_info or _newer(obj, [src] + hdrs):
                jobs.append(ex.submit(_compile_cu, src, obj, verbose or ptxas_info, extra))
        for s in C_SOURCES:
            src, obj = os.path.join(HOST, s), os.path.join(OUT, s + ".o")
            objs.append(obj)
            if force or _newer(obj, [src] + hdrs):
                jobs.append(ex.submit(_compile_c, src, obj, verbose))
        for j in jobs:
            j.result()
    if force or _newer(LIB, objs):
        cuda_lib = os.path.join(CUDA_HOME, "lib64")
        tmp = LIB + ".tmp"
        _run(["g++", "-shared", "-o", tmp, *objs, f"-L{cuda_lib}", "-lcufft", "-lcusparse", "-lcudart",
              f"-Wl,-rpath,{cuda_lib}"], verbose)
        os.replace(tmp, LIB)
    host_objs = [os.path.join(OUT, s + ".o") for s in C_SOURCES]
    if force or _newer(HOST_LIB, host_objs):
        _run(["gcc", "-shared", "-o", HOST_LIB, *host_objs, "-lm"], verbose)
    refabi_src = os.path.join(HOST, "csem_refabi.c")
    if force or _newer(REFABI, [refabi_src, LIB] + hdrs):
        _run(["gcc", "-O3", "-fPIC", "-ffp-contract=off", "-std=gnu99", "-Wall", "-shared", "-I", INCLUDE, refabi_src,
              "-o", REFABI, f"-L{OUT}", "-lcsem_gpu", f"-Wl,-rpath,{OUT}"], verbose)
    drv_src = [os.path.join(HOST, s) for s in DRIVER_SOURCES]
    if all(os.path.exists(s) for s in drv_src) and (force or _newer(DRIVER, drv_src + [LIB] + hdrs)):
        _run(["gcc", "-O3", "-ffp-contract=off", "-std=gnu99", "-Wall", "-I", INCLUDE, *drv_src, "-o", DRIVER,
              f"-L{OUT}", "-lcsem_gpu", f"-Wl,-rpath,{OUT}", "-lm"], verbose)
    return LIB


def clean() -> None:
    shutil.rmtree(OUT, ignore_errors=True)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="--verbose" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
