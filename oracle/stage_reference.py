"""Stages the reference implementation into baseline/_ref/ (git-ignored), laid
out as an installed package, so that machines without the reference tree can
build and run it.

TEST INFRASTRUCTURE ONLY.  The reference's own build system (meson-python) is
not available offline, so `pip install --target baseline/_ref <reference>`
cannot run; instead this copies, unmodified,

    <reference>/fastfermion/*.py   -> baseline/_ref/fastfermion/
    <reference>/src, test, examples -> baseline/_ref/_src/
    pybind11's headers             -> baseline/_ref/_pybind11/include/

and `make -f oracle/ref.mk install` then compiles the reference's pybind11
module from baseline/_ref/_src/src into baseline/_ref/fastfermion/ (its
installed location).  The reference tree is FFG_REFERENCE_SRC (default
/root/reference); nothing is done when it is absent.
"""
import os
import shutil
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DEST = os.path.join(ROOT, "baseline", "_ref")


def _copytree(src, dst):
    if os.path.isdir(dst):
        shutil.rmtree(dst)
    shutil.copytree(src, dst, ignore=shutil.ignore_patterns("__pycache__", "*.so", "*.pyc"))


def stage(ref=None, quiet=True):
    ref = ref or os.environ.get("FFG_REFERENCE_SRC", "/root/reference")
    if not os.path.isdir(os.path.join(ref, "src")):
        return False
    try:
        import pybind11
    except ImportError:
        return False
    stamp = os.path.join(DEST, ".staged")
    newest = max(os.path.getmtime(os.path.join(dp, f)) for dp, _, fs in os.walk(os.path.join(ref, "src"))
                 for f in fs)
    if os.path.exists(stamp) and os.path.getmtime(stamp) >= newest:
        return True
    os.makedirs(DEST, exist_ok=True)
    pkg = os.path.join(DEST, "fastfermion")
    os.makedirs(pkg, exist_ok=True)
    for f in os.listdir(os.path.join(ref, "fastfermion")):
        if f.endswith(".py"):
            shutil.copy2(os.path.join(ref, "fastfermion", f), os.path.join(pkg, f))
    for sub in ("src", "test", "examples"):
        _copytree(os.path.join(ref, sub), os.path.join(DEST, "_src", sub))
    _copytree(pybind11.get_include(), os.path.join(DEST, "_pybind11", "include"))
    open(stamp, "w").write(ref + "\n")
    if not quiet:
        print(f"staged {ref} into {DEST}")
    return True


if __name__ == "__main__":
    ok = stage(sys.argv[1] if len(sys.argv) > 1 else None, quiet=False)
    sys.exit(0 if ok else 1)
