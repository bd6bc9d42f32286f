"""In-tree build of the native parts.

* libcafe_gpu.so: the CUDA engine (csrc/cafe_host.cu, which includes
  csrc/cafe_kernels.cu), compiled by nvcc for sm_103a only, with FP
  contraction off in device (--fmad=false) and host (-ffp-contract=off) code.
* oracle/_build/libcafe_oracle.so: the CPU checker used by tests and the CPU
  baseline (g++).
* oracle/_ref/: the reference built from its own sources with single-rank
  shims, only where the reference checkout is present.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIB_DIR, "libcafe_gpu.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "libcafe_oracle.so")
# the reference checkout's src/src-mpi: CAFE_REF_SRC, else a checkout named
# "reference" beside the repository
REF_SRC = os.environ.get("CAFE_REF_SRC") or os.path.normpath(os.path.join(ROOT, "..", "reference", "src", "src-mpi"))

NVCC_FLAGS = ["-std=c++17", "-O3", "--fmad=false", "-lineinfo",
              "-gencode", "arch=compute_103a,code=sm_103a",
              "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fPIC", "-shared"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cuh", ".h"))] + [os.path.join(ROOT, "include", "cafe_gpu.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_engine(force=False, verbose=False):
    os.makedirs(LIB_DIR, exist_ok=True)
    if not force and not _stale(LIB, _sources()):
        return LIB
    cmd = [_nvcc()] + NVCC_FLAGS + [os.path.join(CSRC, "cafe_host.cu"), os.path.join(CSRC, "cafe_noalloc.cu"),
                                    os.path.join(CSRC, "cafe_batch.cu"), os.path.join(CSRC, "cafe_adjoint.cu"),
                                    "-o", LIB + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def build_oracle(verbose=False):
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "oracle"], check=True,
                   stdout=None if verbose else subprocess.DEVNULL)
    if os.path.isdir(REF_SRC):
        subprocess.run(["make", "-s", "-j4", "-C", ORACLE_DIR, "ref", "REF_SRC=" + REF_SRC], check=True,
                       stdout=None if verbose else subprocess.DEVNULL)
    return ORACLE_LIB


def build(force=False, verbose=False):
    build_engine(force=force, verbose=verbose)
    build_oracle(verbose=verbose)


if __name__ == "__main__":
    build(verbose=True)
