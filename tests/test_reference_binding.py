"""The reference's own Python package and its own tests, with the GPU underneath
its `propagate` through the drop-in module ffcore_gpu
(fastfermion_gb300/binding/ffcore_gpu.cpp, built against the reference's
headers).  The reference is the copy staged in baseline/_ref (built there from
its own sources by oracle/ref.mk); the tests are skipped where it is absent.

Each reference test file compares two calls of propagate; the routing plugin
(tests/refplugin/ffg_ref_route.py) sends one of the two to the GPU and the
other to the reference's CPU code, so the reference's assertions compare the
GPU with the reference itself: omp_test.py and sharded_test.py (n_threads > 1
on the GPU against the serial strategy), batched_test.py (batched=True on the
GPU against batched=False), majorana_circuit_test.py (every propagate call on
the GPU, against the test's own gate-by-gate algorithms).
"""
import glob
import json
import os
import subprocess
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STAGE = os.path.join(ROOT, "baseline", "_ref")
TESTS = os.path.join(STAGE, "_src", "test")
BINDING = os.path.join(ROOT, "fastfermion_gb300", "binding")


def _available():
    return (glob.glob(os.path.join(STAGE, "fastfermion", "ffcore*.so")) and
            glob.glob(os.path.join(BINDING, "ffcore_gpu*.so")) and os.path.isdir(TESTS))


pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not _available(), reason="reference not staged or ffcore_gpu not built")]


def _env(route, counts):
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([STAGE, os.path.join(ROOT, "tests", "refplugin"), BINDING,
                                         env.get("PYTHONPATH", "")])
    env["FFG_REF_ROUTE"] = route
    env["FFG_REF_COUNTS"] = counts
    return env


@pytest.mark.parametrize("files,route", [(["omp_test.py", "sharded_test.py"], "threads"),
                                         (["batched_test.py"], "batched"),
                                         (["majorana_circuit_test.py"], "all")],
                         ids=["omp+sharded", "batched", "majorana_circuit"])
def test_reference_suite_with_gpu_propagate(files, route):
    with tempfile.TemporaryDirectory() as d:
        counts = os.path.join(d, "counts.json")
        r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "ffg_ref_route", "-p", "no:cacheprovider",
                            *files], cwd=TESTS, env=_env(route, counts), capture_output=True, text=True,
                           timeout=900)
        assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
        c = json.load(open(counts))
    assert c["gpu"] > 0, c


def test_reference_example_known_answer_on_gpu():
    """examples/pauli_propagation.py (su4circuit-16, Z15) with maxdegree=4 as a
    keyword: <O> = 0.008664 within 1e-6, and the GPU's terms equal the
    reference CPU's, coefficient for coefficient."""
    script = r'''
import sys, json
sys.path.insert(0, "EXAMPLES")
from common import read_circuit
import fastfermion as ff, ffcore_gpu
circ = read_circuit("EXAMPLES/data/su4circuit-16.txt")
obs = ff.poly("Z15")
g = ffcore_gpu.propagate(circ, obs, maxdegree=4)
c = ff.propagate(circ, obs, maxdegree=4)
gt, ct = g.terms, c.terms  # each .terms access builds a dict of every term
same = len(gt) == len(ct) and all(gt.get(k) == v for k, v in ct.items())
print(json.dumps({"n": len(g.terms), "o": g.overlapwithzero().real, "same": same}))
'''.replace("EXAMPLES", os.path.join(STAGE, "_src", "examples"))
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([sys.executable, "-c", script], env=_env("all", os.path.join(d, "c.json")),
                           capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["n"] == 130863 and out["same"]
    assert abs(out["o"] - 0.008664) <= 1e-6
