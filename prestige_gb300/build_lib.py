"""Build recipe for libprestige_gpu.so (the C-ABI CUDA library), compiled for sm_103a only.

Each .cu file is compiled to an object in parallel, then linked into
prestige_gb300/_build/libprestige_gpu.so.  Host code is compiled with -ffp-contract=off so
that host-side constants follow the same operation order as the oracle on every CPU
(x86 here, Arm on the GPU hosts).
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libprestige_gpu.so")
HOST_DIR = os.path.join(HERE, "host")
HOST_LIB = os.path.join(OUT_DIR, "libprestige_host.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fno-strict-aliasing"]


def _nvcc():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(INCLUDE, "prestige_gpu.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(OUT_DIR, os.path.basename(src)[:-3] + ".o")
    if not _stale(obj, [src, __file__] + headers()):
        return obj
    cmd = [_nvcc()] + ARCH + NVCC_FLAGS + ["-I", INCLUDE, "-c", src, "-o", obj + ".tmp"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose:
        sys.stderr.write(r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build_host(force=False):
    """The C++ host layer (prestige_gb300/host): libprestige_host.so, linked to the CUDA library."""
    srcs = [os.path.join(HOST_DIR, f) for f in os.listdir(HOST_DIR) if f.endswith((".cpp", ".hpp"))]
    if not force and not _stale(HOST_LIB, srcs + [LIB, __file__, os.path.join(INCLUDE, "prestige_gpu.h")]):
        return HOST_LIB
    tmp = HOST_LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-o", tmp,
           os.path.join(HOST_DIR, "prestige_host.cpp"), "-L", OUT_DIR, "-lprestige_gpu", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host layer build failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, HOST_LIB)
    return HOST_LIB


def build(force=False, verbose=False):
    """Compile the library (and the C++ host layer) if any source is newer; return the .so path."""
    lib = _build_cuda(force, verbose)
    build_host(force)
    return lib


def _build_cuda(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sources()
    if not force and not _stale(LIB, srcs + headers() + [__file__]):
        return LIB
    if force:
        for f in os.listdir(OUT_DIR):
            if f.endswith(".o"):
                os.remove(os.path.join(OUT_DIR, f))
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
