"""Build the CPU oracle (test infrastructure) into oracle/_build/.

  libfrico_oracle.so   the C++ restatement in frico_oracle.cpp (g++ -O3 -fopenmp)

When the FRICO sources are present (this only happens on a machine that has
the reference checkout), `build_ref()` additionally compiles the reference's
own files in place into oracle/_ref/ (see ref/Makefile).
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "libfrico_oracle.so"
SRC = HERE / "frico_oracle.cpp"
TABLE = HERE.parent / "frico_gb300" / "csrc" / "dunavant_rules.h"


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    h = hashlib.sha256(SRC.read_bytes() + TABLE.read_bytes()).hexdigest()
    stamp = OUT / ".stamp"
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == h:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
           str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(h)
    return LIB


# Where this build recipe looks for the FRICO checkout when FRICO_REFERENCE is unset:
# the read-only mount of the build machine. Machines without it (the GPU hosts) skip
# the reference build and use the committed fixtures.
DEFAULT_REFERENCE = "/root/reference"


def reference_dir() -> Path | None:
    """The FRICO checkout whose sources pin the oracle: $FRICO_REFERENCE, else the
    build machine's mount; None when neither holds FRICO's sources."""
    ref = Path(os.environ.get("FRICO_REFERENCE") or DEFAULT_REFERENCE)
    return ref if (ref / "src" / "quadratures.cpp").exists() else None


def build_ref() -> Path | None:
    """Compile FRICO's own sources (where they lie) into oracle/_ref/, if present."""
    ref = reference_dir()
    if ref is None or not (HERE / "ref" / "Makefile").exists():
        return None
    r = subprocess.run(["make", "-s", "-C", str(HERE / "ref"), f"REF={ref}"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")
    return HERE / "_ref" / "libfrico_ref.so"


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
