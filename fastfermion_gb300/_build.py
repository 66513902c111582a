"""Builds libffg.so (the CUDA propagation library) in-tree with nvcc for sm_103a."""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libffg.so")
SOURCES = ["ffg_engine.cu", "ffg_pauli.cu", "ffg_majorana.cu", "ffg_batch.cu", "ffg_convert.cu", "ffg_noalloc.cu",
           "ffg_sortmerge.cu", "ffg_mlp.cu"]
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


STAGE = os.path.join(os.path.dirname(HERE), "baseline", "_ref")
BINDING_SRC = os.path.join(HERE, "binding", "ffcore_gpu.cpp")


def binding_path():
    import sysconfig
    return os.path.join(HERE, "binding", "ffcore_gpu" + sysconfig.get_config_var("EXT_SUFFIX"))


def build_binding(force=False):
    """Compiles the drop-in module ffcore_gpu (fastfermion's propagate on libffg)
    against the reference headers and pybind11 staged in baseline/_ref; returns
    its path, or None when they are not staged on this machine."""
    import sysconfig
    src_inc = os.path.join(STAGE, "_src", "src")
    pyb_inc = os.path.join(STAGE, "_pybind11", "include")
    if not (os.path.isdir(src_inc) and os.path.isdir(pyb_inc)):
        return None
    out = binding_path()
    lib = build()
    deps = [BINDING_SRC, lib, os.path.join(os.path.dirname(HERE), "include", "ffg.h")]
    if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cmd = ["g++", "-O3", "-std=c++20", "-shared", "-fPIC", "-fopenmp", "-DFF_OPENMP", '-DFF_VERSION="ref"',
           "-ffp-contract=off", "-w", f"-I{src_inc}", f"-I{os.path.join(src_inc, 'hashmap')}", f"-I{pyb_inc}",
           f"-I{sysconfig.get_paths()['include']}", f"-I{os.path.join(os.path.dirname(HERE), 'include')}",
           BINDING_SRC, f"-L{HERE}", "-lffg", "-Wl,-rpath,$ORIGIN/..", "-o", out + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    import sys
    build(force=True, verbose="-v" in sys.argv)
    print(LIB)
