"""Builds libffg.so (the CUDA propagation library) in-tree with nvcc for sm_103a."""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libffg.so")
SOURCES = ["ffg_engine.cu", "ffg_noalloc.cu", "ffg_sortmerge.cu", "ffg_mlp.cu"]
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
    """Compile libffg.so unless it is up to date (translation units in
    parallel, then one link); returns its path."""
    if not force and not _stale():
        return LIB
    extra = os.environ.get("FFG_BUILD_FLAGS", "").split()
    common = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", *extra,
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(os.path.dirname(HERE), "include")]
    if verbose:
        common.insert(1, "-Xptxas=-v")
    objs, procs = [], []
    for src in SOURCES:
        obj = os.path.join(CSRC, src[:-3] + ".o")
        objs.append(obj)
        procs.append(subprocess.Popen([*common, "-c", os.path.join(CSRC, src), "-o", obj]))
    codes = [p.wait() for p in procs]
    if any(codes):
        raise subprocess.CalledProcessError(next(c for c in codes if c), "nvcc")
    subprocess.run([nvcc(), *ARCH, "-shared", *objs, "-o", LIB + ".tmp"], check=True)
    for o in objs:
        os.remove(o)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    import sys
    build(force=True, verbose="-v" in sys.argv)
    print(LIB)
