"""Build libfrico_gpu.so in-tree (frico_gb300/_lib/) with nvcc for sm_103a.

Translation units compile in parallel; the link is `nvcc -shared`. A stamp of
the source hashes skips the build when nothing changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
BUILD = PKG / "_build"
LIB = LIBDIR / "libfrico_gpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-I", str(ROOT / "include"), "-I", str(CSRC)]
SOURCES = ["api.cu", "fill.cu", "lu.cu", "trsv.cu", "gemm_tc.cu", "lu_nopiv.cu", "fields.cu", "fields_multi.cu", "sweep.cu", "adjoint.cu", "gmres.cu", "fields_gemm.cu",
           "mesh_host.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stamp() -> str:
    h = hashlib.sha256()
    for f in sorted(CSRC.glob("*")) + [ROOT / "include" / "frico_gpu.h", Path(__file__)]:
        if f.is_file():
            h.update(f.name.encode())
            h.update(f.read_bytes())
    return h.hexdigest()


def build(verbose: bool = False, force: bool = False) -> Path:
    stamp_file = LIBDIR / ".stamp"
    stamp = _stamp()
    if not force and LIB.exists() and stamp_file.exists() and stamp_file.read_text() == stamp:
        return LIB
    LIBDIR.mkdir(exist_ok=True)
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src: str) -> Path:
        obj = BUILD / (src + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
        if src.endswith(".cpp"):
            cmd = [nvcc, *NVCC_FLAGS, "-x", "c++", "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp_file.write_text(stamp)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
