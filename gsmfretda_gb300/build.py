"""Build libgpda.so in-tree for sm_103a (no cmake, one -gencode, parallel TUs).

    python -m gsmfretda_gb300.build

-fmad=false: no multiply-add is contracted unless written as fmaf(), so every
FP32 sampling decision rounds exactly where the host restatement rounds.
-ffp-contract=off does the same for the host-side parameter derivation.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgpda.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["gpda_kernels.cu", "gpda_engine.cu", "gpda_mc.cu", "gpda_params.cpp", "gpda_noalloc.cu",
           "gpda_expected.cu"]
HEADERS = ["gpda_device.cuh", "gpda_internal.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
           "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
           "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA extension cannot be built")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] + \
           [os.path.join(INCLUDE, "gpda.h")]
    if not _stale(obj, deps):
        return obj
    lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
    cmd = [nvcc()] + ARCH + NVFLAGS + ["-I", INCLUDE, "-c"] + lang + [os.path.join(CSRC, src), "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def ptxas_report() -> str:
    """Register / spill / shared-memory usage of the kernels (-Xptxas -v)."""
    cmd = [nvcc()] + ARCH + NVFLAGS + ["-Xptxas", "-v", "-I", INCLUDE, "-c", "-x", "cu",
                                       os.path.join(CSRC, "gpda_kernels.cu"), "-o", os.devnull]
    return subprocess.run(cmd, capture_output=True, text=True, check=True).stderr


if __name__ == "__main__":
    print(build(verbose=True))
    if "--ptxas" in sys.argv:
        print(ptxas_report())
