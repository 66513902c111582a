"""The C++ binding shown in INTEGRATION.md compiles against the reference's own
headers and include/ffg.h (syntax and type check only; skipped where the
reference sources are not present)."""
import os
import re
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("FFG_REFERENCE_SRC", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")) or shutil.which("g++") is None,
                    reason="reference sources not available")
def test_integration_snippet_compiles():
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", doc, flags=re.S)
    assert blocks, "no C++ block in INTEGRATION.md"
    src = ('#include "pauli/propagate.h"\nusing namespace fastfermion;\n' + blocks[0] +
           "\nint main() { return 0; }\n")
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "shim.cpp")
        open(f, "w").write(src)
        r = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", "-w", f"-I{REF}/src",
                            f"-I{REF}/src/hashmap", f"-I{ROOT}/include", f], capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stderr[-3000:]
