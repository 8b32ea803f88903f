"""Regenerates tests/golden/cpp_format.txt: a seeded list of doubles (EM-sized
values, integers, powers of ten, extremes) formatted by std::format("{}", x),
the way FRICO's text outputs print doubles. Needs g++ with C++20 <format>."""
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def values():
    rng = np.random.default_rng(20260103)
    v = [0.0, -0.0, 1.0, -1.0, 0.1, 0.5, 2.5, 3e8, 4.5e8, 1e16, 1e15, 1e17, 1e21, 1e-4, 1e-5, 1e-300, 5e-324,
         1.7976931348623157e308, 65535.0, 123456789012.0, 12345678.9, 1 / 3, 2 / 3, 75.08853312, 50.0]
    v += list(10.0 ** rng.uniform(-12, 12, 600) * rng.choice([-1, 1], 600))
    v += list(np.round(rng.uniform(-1e6, 1e6, 100)))
    v += list(rng.uniform(0, 1, 100))
    v += [float(10.0 ** e) for e in range(-20, 23)]
    v += list(200e6 + np.arange(256) * 600e6 / 255)
    return [float(x) for x in v]


def main():
    src = HERE / "cpp_format_golden.cpp"
    with tempfile.TemporaryDirectory() as td:
        exe = Path(td) / "fmt"
        subprocess.run(["g++", "-std=c++23", "-O1", str(src), "-o", str(exe)], check=True)
        inp = "\n".join(x.hex() for x in values()) + "\n"
        out = subprocess.run([str(exe)], input=inp, capture_output=True, text=True, check=True).stdout
    (HERE / "cpp_format.txt").write_text(out)
    print(f"wrote {len(out.splitlines())} lines", file=sys.stderr)


if __name__ == "__main__":
    main()
