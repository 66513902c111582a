"""pytest plugin that runs the reference's own test files with the GPU under
fastfermion.propagate (the drop-in module ffcore_gpu).

FFG_REF_ROUTE selects which calls go to the GPU, so that each test compares
the GPU with the reference's own CPU path instead of with itself:
  threads  calls with n_threads > 1 (omp_test.py, sharded_test.py compare them
           with the serial strategy);
  batched  calls with batched=True (batched_test.py compares them with
           batched=False);
  all      every call (tests that compare with an independent algorithm);
  none     no call (checks the plumbing on machines without a GPU).
The number of calls on each side is written to FFG_REF_COUNTS as JSON.  The
reference's test/common.py imports openfermion, which the tests run here do not
call (it names three of its classes in annotations); a stand-in module with
those names is used when it is not installed.
"""
import json
import os
import sys
import types

_counts = {"gpu": 0, "cpu": 0}


def pytest_configure(config):
    import fastfermion  # before the stand-in: the package's optional openfermion adapter stays off
    try:
        import openfermion  # noqa: F401
    except ImportError:
        stub = types.ModuleType("openfermion")
        for name in ("QubitOperator", "FermionOperator", "MajoranaOperator"):  # only named in annotations
            setattr(stub, name, type(name, (), {}))
        sys.modules["openfermion"] = stub
    mode = os.environ.get("FFG_REF_ROUTE", "all")
    cpu = fastfermion.propagate
    gpu = None
    if mode != "none":
        import ffcore_gpu
        gpu = ffcore_gpu.propagate

    def propagate(circuit, observable, *args, **kw):
        n_threads = args[0] if args else kw.get("n_threads", 1)
        batched = kw.get("batched", True)
        use = {"threads": isinstance(n_threads, int) and n_threads > 1, "batched": batched is True,
               "all": True, "none": False}[mode]
        _counts["gpu" if use else "cpu"] += 1
        return (gpu if use else cpu)(circuit, observable, *args, **kw)

    fastfermion.propagate = propagate


def pytest_unconfigure(config):
    path = os.environ.get("FFG_REF_COUNTS")
    if path:
        with open(path, "w") as f:
            json.dump(_counts, f)
