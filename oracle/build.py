"""Build recipe for the CPU oracle (test infrastructure only).

    python oracle/build.py        # -> oracle/liboracle.so

The reference itself cannot be compiled here (xtensor, CLI11, HighFive and
pugixml are not installed), so oracle/_ref stays empty.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def build(verbose=False):
    src = os.path.join(HERE, "oracle_capi.cpp")
    hdr = os.path.join(HERE, "samurai_oracle.hpp")
    out = os.path.join(HERE, "liboracle.so")
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(src), os.path.getmtime(hdr), os.path.getmtime(__file__)):
        return out
    # -O3 with FP contraction off (the reference's non-contracting build); no -march=native: the same
    # source builds on x86-64 and on the aarch64 GPU hosts and must round identically on both
    cmd = ["g++", "-std=c++20", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-o", out + ".tmp", src]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
