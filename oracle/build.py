"""Build recipe for the CPU oracle (test infrastructure): oracle/_build/liboracle.so.

The oracle is compiled with -ffp-contract=off so that its operation order is the
definition of the method (no fused multiply-add contraction), and with OpenMP over the
target particle so its results do not depend on the thread count.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "oracle_capi.cpp")]
HEADERS = [os.path.join(HERE, "prestige_oracle.hpp")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SOURCES + HEADERS + [__file__])


def build(force=False):
    """Compile liboracle.so if it is missing or older than its sources; return its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", tmp] + SOURCES
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
