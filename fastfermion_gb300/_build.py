"""Builds libffg.so (the CUDA propagation library) in-tree with nvcc for sm_103a."""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libffg.so")
SOURCES = ["ffg_engine.cu", "ffg_noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libffg")
    return exe


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "ffg.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    """Compile libffg.so unless it is up to date; returns its path."""
    if not force and not _stale():
        return LIB
    extra = os.environ.get("FFG_BUILD_FLAGS", "").split()
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", *extra,
           "-Xcompiler", "-fPIC,-ffp-contract=off", "-shared",
           "-I", os.path.join(os.path.dirname(HERE), "include"),
           *[os.path.join(CSRC, s) for s in SOURCES], "-o", LIB + ".tmp"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    import sys
    build(force=True, verbose="-v" in sys.argv)
    print(LIB)
