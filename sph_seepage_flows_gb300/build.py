"""In-tree build of the CUDA library libsf_gb300.so (sm_103a) and of the C++
drop-in facade test program.

Each translation unit is compiled by nvcc in parallel into _build/, then
linked into sph_seepage_flows_gb300/libsf_gb300.so. The passes whose results
are bit-exact against the reference (sort, density, average flow, voidage /
adhesion, integrate) are built with --fmad=false and IEEE division / square
root so that their FP32 arithmetic matches the reference kernels' operation
order exactly; the adjoint (sf_adjoint.cu) uses the fast intrinsics.
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
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libsf_gb300.so")
SOURCES = ["sf_kernels.cu", "sf_momentum.cu", "sf_sort.cu", "sf_adjoint.cu", "sf_capi.cu", "sf_noalloc.cu", "sf_bgeo.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = os.path.join(cuda, "bin", "nvcc")
    return exe if os.path.exists(exe) else (shutil.which("nvcc") or "nvcc")


# The forward passes reproduce the reference's FP32 operation order (no
# contraction, IEEE division and square root). The adjoint only has to be
# accurate to its gradient tolerance and uses the fast intrinsics. The
# momentum passes (sf_momentum.cu) keep the forward arithmetic too: with
# multiply-add contraction the compiler contracts the list walk and the
# overflow stencil walk, into which the same pair term is inlined, in
# different places, so a particle's force would depend on which path ran.
PRECISE = ["--fmad=false", "-prec-div=true", "-prec-sqrt=true"]
FAST_SOURCES = {"sf_adjoint.cu"}


def arith_flags(src: str) -> list:
    return ["-use_fast_math"] if src in FAST_SOURCES else PRECISE


def common_flags(src: str = "") -> list:
    arith = arith_flags(src)
    return ARCH + ["-O3", "-std=c++17", "-lineinfo"] + arith + [
        "--extended-lambda", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", os.path.join(ROOT, "include")]


def _compile(src: str, extra: list) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + common_flags(src) + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def _stale(target: str, deps: list) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, verbose: bool = False, extra: list | None = None) -> str:
    """Compile and link libsf_gb300.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "sf_capi.h")]
    if not force and not _stale(LIB, deps):
        return LIB
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


def ptxas_report(src: str = "sf_kernels.cu") -> str:
    """-Xptxas -v resource usage of one translation unit (registers, spills)."""
    os.makedirs(BUILD, exist_ok=True)
    cmd = [nvcc()] + common_flags(src) + ["-Xptxas", "-v", "-c", os.path.join(CSRC, src), "-o",
                                       os.path.join(BUILD, "ptxas_probe.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.stdout + r.stderr


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "ptxas":
        print(ptxas_report(*(sys.argv[2:] or [])))
    else:
        print(build_library(force="-f" in sys.argv, verbose=True))
