"""Builds libnbg_cuda.so (sm_103a) in-tree, under nbodygradient.jl_gb300/_build/.

The library is one host/orchestration unit (csrc/nbg_cuda.cu), the request
server (csrc/nbg_server.cu), the initial conditions (csrc/nbg_ics.cu), the fixed scratch area of the allocation-free
entry point (csrc/nbg_noalloc.cu), and one
kernel-instantiation unit per body count (csrc/nbg_inst.cu with -DNBG_N=2..10);
the units compile in parallel and are linked with nvcc -shared.  A content
hash of the sources and flags skips the build when nothing changed.
"""
import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libnbg_cuda.so"
LIB_PATH = os.path.join(BUILD_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: scalar products and sums round one by one as in Julia; the
# kernels call fma() where a fused product is meant.  -ffp-contract=off does
# the same for the host code (step counts, s.t), which GCC would otherwise
# contract on AArch64.
NVCC_FLAGS = ARCH + ["-O3", "--fmad=false", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE]
BODY_COUNTS = list(range(2, 11))


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: set NVCC or put the CUDA toolkit on PATH")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h", ".hpp"))) + \
        [os.path.join(INCLUDE, "nbg.h")]


def _digest():
    h = hashlib.sha256()
    for p in _sources():
        with open(p, "rb") as f:
            h.update(os.path.basename(p).encode())
            h.update(f.read())
    h.update(" ".join(NVCC_FLAGS).encode())
    return h.hexdigest()


def build(force=False, verbose=False, jobs=None):
    """Compile and link libnbg_cuda.so; returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    stamp = os.path.join(BUILD_DIR, "stamp.txt")
    dig = _digest()
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == dig:
                return LIB_PATH
    nv = nvcc()
    units = [(os.path.join(CSRC, "nbg_cuda.cu"), os.path.join(BUILD_DIR, "nbg_cuda.o"), []),
             (os.path.join(CSRC, "nbg_noalloc.cu"), os.path.join(BUILD_DIR, "nbg_noalloc.o"), []),
             (os.path.join(CSRC, "nbg_server.cu"), os.path.join(BUILD_DIR, "nbg_server.o"), []),
             (os.path.join(CSRC, "nbg_ics.cu"), os.path.join(BUILD_DIR, "nbg_ics.o"), []),
             (os.path.join(CSRC, "nbg_batch_async.cu"), os.path.join(BUILD_DIR, "nbg_batch_async.o"), [])]
    for n in BODY_COUNTS:
        units.append((os.path.join(CSRC, "nbg_inst.cu"), os.path.join(BUILD_DIR, "nbg_inst_%d.o" % n),
                      ["-DNBG_N=%d" % n]))

    def compile_one(u):
        src, obj, extra = u
        cmd = [nv] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed (%s):\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return obj

    jobs = jobs or min(len(units), max(1, os.cpu_count() or 1))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = LIB_PATH + ".tmp"
    cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed (%s):\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as f:
        f.write(dig)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
