"""The FRICO-side adapter integration/emw_gpu_backend.cpp (the file a maintainer
adds to FRICO) compiles against FRICO's own headers (src/emw_solver.h,
src/emw_postpro_common.h) and include/frico_gpu.h, with the shims and flags the
oracle uses to compile FRICO's sources (oracle/ref/Makefile); INTEGRATION.md
quotes that file verbatim. The compile check is skipped where the FRICO
checkout or g++ is absent."""
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
ADAPTER = ROOT / "integration" / "emw_gpu_backend.cpp"


def test_integration_doc_quotes_the_adapter():
    blocks = re.findall(r"```cpp\n(.*?)```", (ROOT / "INTEGRATION.md").read_text(), re.S)
    assert ADAPTER.read_text() in blocks


def test_adapter_compiles_against_frico_headers():
    import build as oracle_build
    ref = oracle_build.reference_dir()
    if ref is None or not (ref / "src" / "emw_solver.h").exists() or shutil.which("g++") is None:
        pytest.skip("FRICO checkout or g++ not available")
    shim = ROOT / "oracle" / "ref"
    cmd = ["g++", "-std=c++23", "-fsyntax-only", "-w", "-DHAVE_LAPACK", "-include", str(shim / "lapack_rename.h"),
           "-I", str(shim / "shim"), "-I", str(ref / "src"), "-I", str(ROOT / "include"), str(ADAPTER)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
