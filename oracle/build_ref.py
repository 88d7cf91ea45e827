"""Compile the reference's own binomial sampler (src/binom.cuh, read from the
reference tree where it lies) into oracle/_ref/libref_binom.so.

TEST INFRASTRUCTURE ONLY. Used to pin the oracle's binomial sampler against
the reference's and to generate tests/golden/ref_binomial.npz. The reference
tree exists only where it is mounted; elsewhere the committed golden fixture
stands in for it.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree's mount point (GPDA_REFERENCE overrides it), as in build_mcref.py
REF_SRC = os.path.join(os.environ.get("GPDA_REFERENCE", "/root/reference"), "src")
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_binom.so")


def available() -> bool:
    return os.path.exists(os.path.join(REF_SRC, "binom.cuh"))


def build() -> str:
    if os.path.exists(LIB):
        return LIB
    if not available():
        raise FileNotFoundError(f"{REF_SRC}/binom.cuh not present")
    os.makedirs(OUT_DIR, exist_ok=True)
    cuh = os.path.join(REF_SRC, "binom.cuh")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f'-DREF_BINOM_CUH="{cuh}"',
           os.path.join(HERE, "ref_binom_wrap.cpp"), "-o", LIB + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build())
