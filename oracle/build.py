"""Build recipe for the CPU oracle (test infrastructure): oracle/_build/liboracle.so and the
CPU timing build oracle/_build/liboracle_timing.so.

The oracle is compiled with -ffp-contract=off so that its operation order is the
definition of the method (no fused multiply-add contraction), and with OpenMP over the
target particle so its results do not depend on the thread count.

The timing build (cpu_timing.cpp: cell-sorted arrays, neighbour lists built once per step,
a parallel radix sort) is the CPU baseline that bench.py times.  It is compiled with
contraction allowed and -funroll-loops, for speed.  It is not built with -march=native: the
same recipe must build on the x86 development container and on the Arm GPU host, and on the
Arm host (Neoverse V2, whose SVE vectors are 128 bits wide) the default target's 128-bit NEON
vectors are as wide.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
TIMING_LIB = os.path.join(OUT_DIR, "liboracle_timing.so")
SOURCES = [os.path.join(HERE, "oracle_capi.cpp")]
TIMING_SOURCES = [os.path.join(HERE, "cpu_timing.cpp")]
HEADERS = [os.path.join(HERE, "prestige_oracle.hpp")]

FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off"]
TIMING_FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=fast", "-funroll-loops"]


def _stale(lib, sources):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(p) > t for p in sources + HEADERS + [__file__])


def _compile(lib, sources, flags):
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = lib + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++"] + flags + ["-fPIC", "-shared", "-o", tmp] + sources)
    os.replace(tmp, lib)


def build(force=False):
    """Compile liboracle.so if it is missing or older than its sources; return its path."""
    if force or _stale(LIB, SOURCES):
        _compile(LIB, SOURCES, FLAGS)
    return LIB


def build_timing(force=False):
    """Compile the CPU timing build (liboracle_timing.so) if needed; return its path."""
    if force or _stale(TIMING_LIB, TIMING_SOURCES):
        _compile(TIMING_LIB, TIMING_SOURCES, TIMING_FLAGS)
    return TIMING_LIB


if __name__ == "__main__":
    print(build(force=True))
    print(build_timing(force=True))
