"""Build the reference-kernel harness (oracle/mcref_harness.cu) into
oracle/_ref/libmcref.so. TEST INFRASTRUCTURE ONLY.

Two steps, each where it can run:

  extract()  where the reference tree is mounted: copies the text of
             mc_kernel (src/mc.cu, from its `__global__ void mc_kernel(` to
             the matching closing brace) into oracle/_ref/mcref/mc_kernel.inc
             and src/gen_rand.cuh, src/binom.cuh beside it, and the reference's
             GPU thread (src/gpuWorker.cpp, .hpp) into oracle/_ref/worker/ for
             tests/test_ref_worker.py. oracle/_ref/ is
             git-ignored (nothing of the reference is committed) and travels
             with the working tree to the GPU machine.
  build()    wherever oracle/_ref/mcref/ exists and nvcc is present: compiles
             the harness for sm_103a against those files, linking cuRAND
             (the reference's own RNG set-up needs its direction vectors).

The rest of src/mc.cu (the mc class) needs Eigen, Boost and the reference's
own headers and is not built; the kernel uses Eigen only through one
column-major accessor, which the harness supplies.
"""
import os
import re
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree's mount point (GPDA_REFERENCE overrides it)
REF_ROOT = os.environ.get("GPDA_REFERENCE", "/root/reference")
OUT_DIR = os.path.join(HERE, "_ref")
SRC_DIR = os.path.join(OUT_DIR, "mcref")
# the reference's GPU thread (src/gpuWorker.{cpp,hpp}), compiled by
# tests/test_ref_worker.py against the drop-in header
WORKER_DIR = os.path.join(OUT_DIR, "worker")
WORKER_FILES = ("gpuWorker.cpp", "gpuWorker.hpp")
LIB = os.path.join(OUT_DIR, "libmcref.so")
HARNESS = os.path.join(HERE, "mcref_harness.cu")
FILES = ("mc_kernel.inc", "gen_rand.cuh", "binom.cuh")


def kernel_text(mc_cu: str) -> str:
    """mc_kernel's definition: its signature and body, braces matched outside
    comments and string literals."""
    m = re.search(r"__global__\s+void\s+mc_kernel\s*\(", mc_cu)
    if not m:
        raise ValueError("mc_kernel not found")
    depth, j, n = 0, m.end(), len(mc_cu)
    while j < n:
        if mc_cu.startswith("//", j):
            j = mc_cu.find("\n", j)
            j = n if j < 0 else j
        elif mc_cu.startswith("/*", j):
            j = mc_cu.index("*/", j) + 1
        elif mc_cu[j] in "\"'":
            q = mc_cu[j]
            j += 1
            while mc_cu[j] != q:
                j += 2 if mc_cu[j] == "\\" else 1
        elif mc_cu[j] == "{":
            depth += 1
        elif mc_cu[j] == "}":
            depth -= 1
            if depth == 0:
                return mc_cu[m.start():j + 1] + "\n"
        j += 1
    raise ValueError("unbalanced braces in mc_kernel")


def extract() -> bool:
    src = os.path.join(REF_ROOT, "src")
    if not os.path.exists(os.path.join(src, "mc.cu")):
        return False
    os.makedirs(SRC_DIR, exist_ok=True)
    with open(os.path.join(src, "mc.cu")) as f:
        text = kernel_text(f.read())
    with open(os.path.join(SRC_DIR, "mc_kernel.inc"), "w") as f:
        f.write(text)
    for name in ("gen_rand.cuh", "binom.cuh"):
        shutil.copyfile(os.path.join(src, name), os.path.join(SRC_DIR, name))
    os.makedirs(WORKER_DIR, exist_ok=True)
    for name in WORKER_FILES:
        shutil.copyfile(os.path.join(src, name), os.path.join(WORKER_DIR, name))
    return True


def available() -> bool:
    return all(os.path.exists(os.path.join(SRC_DIR, f)) for f in FILES)


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build(verbose: bool = False, out: str = LIB, fmad: bool = False) -> str:
    """The harness compiled with -fmad=false by default: every FP32 expression
    of mc_kernel rounds as its source text is written (nvcc's default
    contraction would fuse, e.g., f_if = (gamma - Dch2Ach) * f_id +
    (1 - DexDirAem) * f_ia into one fused multiply-add, a compiler choice
    that moves the sum by an ulp; the reference's CMake build leaves the
    default on)."""
    extract()
    if not available():
        raise FileNotFoundError(f"{SRC_DIR}: the reference kernel sources were not extracted")
    deps = [HARNESS] + [os.path.join(SRC_DIR, f) for f in FILES]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cmd = [nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
           f"-fmad={'true' if fmad else 'false'}", "-Xcompiler", "-fPIC", "-w", "-I", SRC_DIR,
           HARNESS, "-o", out + ".tmp", "-lcurand"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build(verbose=True))
