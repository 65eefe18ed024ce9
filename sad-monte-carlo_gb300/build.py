"""Build recipe for libsadmc_gb300.so (CUDA kernels for sm_103a + the C ABI host layer).

Compiles every translation unit under csrc/ in parallel with nvcc and links one shared
library in lib/.  -fmad=false keeps a*b+c un-fused so the FP64 bookkeeping rounds like
the FP64 oracle; the binary32 hot loops use explicit __fmaf_rn where they want fusion.
"""
import concurrent.futures
import hashlib
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libsadmc_gb300.so")
STAMP = os.path.join(LIBDIR, "build.stamp")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsadmc_gb300")
    return p


def _sources():
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    hdrs = sorted(f for f in os.listdir(CSRC) if f.endswith((".cuh", ".h")))
    return srcs, hdrs


def _digest():
    srcs, hdrs = _sources()
    h = hashlib.sha256()
    h.update(platform.machine().encode())
    h.update(" ".join(ARCH + NVFLAGS).encode())
    for f in srcs + hdrs:
        with open(os.path.join(CSRC, f), "rb") as fh:
            h.update(f.encode())
            h.update(fh.read())
    with open(os.path.join(HERE, "..", "include", "sadmc_gpu.h"), "rb") as fh:
        h.update(fh.read())
    return h.hexdigest()


def up_to_date():
    if not (os.path.exists(LIB) and os.path.exists(STAMP)):
        return False
    with open(STAMP) as fh:
        return fh.read().strip() == _digest()


def build(force=False, verbose=False, jobs=None):
    """Compile and link lib/libsadmc_gb300.so unless it is current for this machine."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    srcs, _ = _sources()

    def compile_one(src):
        obj = os.path.join(OBJDIR, src + ".o")
        cmd = [nvcc, "-c", os.path.join(CSRC, src), "-o", obj] + ARCH + NVFLAGS
        if src.endswith(".cpp"):
            cmd = [nvcc, "-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj] + ARCH + NVFLAGS
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, srcs))
    cmd = [nvcc, "-shared", "-o", LIB] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    with open(STAMP, "w") as fh:
        fh.write(_digest())
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
