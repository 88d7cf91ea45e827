"""Build the CPU oracle shared library (test infrastructure only).

    python oracle/build_oracle.py          -> oracle/liborc.so

-ffp-contract=off keeps every FP32 operation rounding where the device code
rounds; no -march flags so that the same source builds on x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def build(verbose: bool = False) -> str:
    src = os.path.join(HERE, "gpda_oracle.c")
    out = os.path.join(HERE, "liborc.so")
    deps = [src, os.path.join(HERE, "gpda_oracle_core.inc"), os.path.join(HERE, "rc_unit_body.inc"),
            os.path.join(HERE, "gpda_oracle.h")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cmd = ["gcc", "-O3", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", "-Wall", "-Wno-unused-function", src, "-o", out + ".tmp", "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
