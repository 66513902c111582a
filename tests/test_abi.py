"""The C-ABI library builds, loads without a GPU and exports every entry point
declared in include/ffg.h; host-side helpers behave as documented."""
import math
import os
import re
import subprocess

import numpy as np
import pytest

from fastfermion_gb300 import _build, _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    txt = open(os.path.join(ROOT, "include", "ffg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ffg_[a-z0-9_]+)\s*\(", txt)))


def test_header_symbols_exported():
    path = _build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r" T (ffg_\w+)", out))
    missing = [s for s in declared() if s not in exported]
    assert not missing, missing
    L = _native.lib()
    for s in declared():
        assert hasattr(L, s)


def test_every_translation_unit_is_built():
    """Every CUDA source of the library is compiled into libffg (the host engine
    is split by entry point over ffg_engine_impl.cuh)."""
    csrc = os.path.join(ROOT, "fastfermion_gb300", "csrc")
    units = sorted(f for f in os.listdir(csrc) if f.endswith(".cu"))
    assert units == sorted(_build.SOURCES), (units, _build.SOURCES)


def test_binding_covers_header():
    assert sorted(_native.EXPORTS) == declared()


def test_sm103a_only():
    """The library carries an sm_103a cubin and no other architecture."""
    out = subprocess.run(["cuobjdump", "--list-elf", _build.build()], capture_output=True,
                         text=True).stdout
    arches = set(re.findall(r"sm_(\d+a?)", out))
    assert arches == {"103a"}, arches


def test_abs_le_matches_libm_hypot():
    """Truncation predicate: hypot(re, im) <= tau as libm rounds it, including
    pairs whose magnitude sits within a few ulps of tau."""
    rng = np.random.default_rng(7)
    for tau in (1e-8, 1e-6, 1e-3, 0.3, 1e-7):
        for _ in range(2000):
            ang = rng.uniform(0, 2 * math.pi)
            r = tau * (1 + rng.integers(-4, 5) * 2.0 ** -52)
            a, b = r * math.cos(ang), r * math.sin(ang)
            assert _native.abs_le(a, b, tau) == (math.hypot(a, b) <= tau), (a, b, tau)
        for _ in range(2000):
            a, b = rng.normal(size=2) * tau * rng.uniform(0.1, 3)
            assert _native.abs_le(a, b, tau) == (math.hypot(a, b) <= tau)
    assert _native.abs_le(1e-9, 0.0, 1e-9) and not _native.abs_le(-1.0000000001e-9, 0.0, 1e-9)
    assert not _native.abs_le(float("nan"), 0.0, 1.0)


def test_schedule_batches_like_reference():
    """Greedy commuting runs, back to front, split at Clifford gates."""
    import fastfermion_gb300 as ff
    c = ff.build_circuit(ff.workloads.kicked_ising_circuit(0.3, 4, 4, 2))
    assert _native.pauli_schedule(ff.encode_pauli_circuit(c)) == [16, 24, 16, 24]
    assert _native.pauli_schedule(ff.encode_pauli_circuit(c), batched=False) == [1] * 80
    c2 = [ff.ROT("X", [0], 0.1), ff.H(1), ff.ROT("Z", [0], 0.2), ff.ROT("Z", [1], 0.3),
          ff.ROT("X", [1], 0.4)]
    assert _native.pauli_schedule(ff.encode_pauli_circuit(c2)) == [1, 2, 1]
