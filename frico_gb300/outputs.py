"""FRICO's text outputs, byte for byte, so that GPU results drop into the
reference's gnuplot scripts (share/gnuplot/*):

  port_sweep.txt        write_sweep_data           src/emw_ana_antenna.cpp:151-172
  polar_<step>.txt      write_radiation_diagrams   src/emw_ana_antenna.cpp:174-204
  bistatic_rcs_<step>.txt                          src/emw_ana_bistatic_rcs.cpp:97-117
  near-field samples    (one line per plane vertex: x y z and |E|, |H|)

FRICO prints doubles with std::println("{}", x): the shortest decimal string
that round-trips, in fixed or scientific notation, whichever is shorter (fixed
on a tie), scientific exponents with a sign and at least two digits.
`cpp_format` reproduces that from Python's shortest round-trip digits.
"""
from __future__ import annotations

import math
import os
from pathlib import Path

import numpy as np


def cpp_format(x: float) -> str:
    """std::format("{}", double)."""
    x = float(x)
    if math.isnan(x):
        return "nan" if math.copysign(1.0, x) > 0 else "-nan"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    if x == 0.0:
        return "-0" if math.copysign(1.0, x) < 0 else "0"
    sign = "-" if x < 0 else ""
    mant, _, exp = repr(abs(x)).partition("e")   # shortest round-trip digits
    ip, _, fp = mant.partition(".")
    digits = ip + fp                             # value = int(digits) * 10^scale
    scale = (int(exp) if exp else 0) - len(fp)
    digits = digits.lstrip("0")
    trailing = len(digits) - len(digits.rstrip("0"))
    digits = digits.rstrip("0")
    scale += trailing
    n = len(digits)
    point = n + scale                            # value = 0.digits * 10^point
    sexp = point - 1
    sci = digits[0] + ("." + digits[1:] if n > 1 else "") + "e" + ("-" if sexp < 0 else "+") + f"{abs(sexp):02d}"
    if point <= 0:
        fix = "0." + "0" * (-point) + digits
    elif point >= n:
        fix = digits + "0" * (point - n)
    else:
        fix = digits[:point] + "." + digits[point:]
    return sign + (fix if len(fix) <= len(sci) else sci)


def _line(*vals) -> str:
    return " ".join(str(v) if isinstance(v, (int, np.integer)) else cpp_format(v) for v in vals)


def write_port_sweep(path, freqs, ports, Z0: float = 50.0) -> None:
    """port_sweep.txt: one line per step {step frequency Re(Z) Im(Z) SWR}."""
    with open(path, "w") as f:
        f.write(f"# Port sweep results, Z0 = {Z0:.1f} Ohm\n")
        f.write("# step  frequency    Re(Z)    Im(Z)    SWR\n")
        for i, (fr, p) in enumerate(zip(freqs, ports)):
            z = complex(p["impedance"])
            f.write(_line(i, float(fr), z.real, z.imag, float(p["swr"])) + "\n")


def write_radiation_diagrams(path, freq: float, gain_xy, gain_yz, gain_xz) -> None:
    """polar_<step>.txt: 360 lines {angle XY_lin XY_dB YZ_lin YZ_dB XZ_lin XZ_dB}."""
    with open(path, "w") as f:
        f.write(f"# FRICO radiation patterns. Frequency = {cpp_format(freq)}\n")
        f.write("# angle XY_lin XY_dB YZ_lin YZ_dB XZ_lin XZ_dB\n")
        for i in range(360):
            a, b, c = float(gain_xy[i]), float(gain_yz[i]), float(gain_xz[i])
            f.write(_line(i, a, _db(a), b, _db(b), c, _db(c)) + "\n")


def _db(g: float) -> float:
    return 10.0 * math.log10(g) if g > 0 else (-math.inf if g == 0 else math.nan)


def write_bistatic_rcs(path, rcs) -> None:
    """bistatic_rcs_<step>.txt: 359 lines {angle VV_theta HH_theta VV_phi HH_phi}."""
    rcs = np.asarray(rcs, np.float64).reshape(359, 4)
    with open(path, "w") as f:
        f.write("# FRICO bistatic RCS computation\n")
        f.write("# Angle, VV_theta, HH_theta, VV_phi, HH_phi\n")
        for i in range(359):
            f.write(_line(i, *rcs[i]) + "\n")


def write_antenna_sweep(outdir, results, Z0: float = 50.0) -> list[Path]:
    """What FRICO's antenna do_sweep writes with text output on
    (src/emw_ana_antenna.cpp:273-283): polar_<step>.txt per step, then
    port_sweep.txt. `results` are AntennaResult items."""
    outdir = Path(outdir)
    os.makedirs(outdir, exist_ok=True)
    paths = []
    for i, r in enumerate(results):
        p = outdir / f"polar_{i}.txt"
        write_radiation_diagrams(p, r.frequency, r.gain_XY, r.gain_YZ, r.gain_XZ)
        paths.append(p)
    p = outdir / "port_sweep.txt"
    write_port_sweep(p, [r.frequency for r in results], [r.port for r in results], Z0)
    paths.append(p)
    return paths


def write_bistatic_sweep(outdir, rcs_per_step) -> list[Path]:
    """bistatic_rcs_<step>.txt per step, as the bistatic do_sweep writes them."""
    outdir = Path(outdir)
    os.makedirs(outdir, exist_ok=True)
    paths = []
    for i, r in enumerate(rcs_per_step):
        p = outdir / f"bistatic_rcs_{i}.txt"
        write_bistatic_rcs(p, r)
        paths.append(p)
    return paths
