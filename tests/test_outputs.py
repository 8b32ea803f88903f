"""Text outputs in FRICO's exact format (CPU): std::format("{}", double) golden
strings from g++, the file layouts of port_sweep / polar / bistatic_rcs, and the
sampling-plane parser and grid."""
from pathlib import Path

import numpy as np
import pytest

from frico_gb300.outputs import (cpp_format, write_antenna_sweep, write_bistatic_rcs, write_port_sweep,
                                 write_radiation_diagrams)
from frico_gb300.sampling import parse_sampling_plane, sampling_plane_points

GOLDEN = Path(__file__).resolve().parent / "golden" / "cpp_format.txt"


def test_cpp_format_matches_std_format_golden():
    lines = GOLDEN.read_text().splitlines()
    assert len(lines) > 1000
    for ln in lines:
        hx, want = ln.split(" ")
        assert cpp_format(float.fromhex(hx)) == want, (hx, want)


def test_cpp_format_special_values():
    assert cpp_format(float("inf")) == "inf" and cpp_format(float("-inf")) == "-inf"
    assert cpp_format(float("nan")) == "nan"


def test_port_sweep_layout(tmp_path):
    p = tmp_path / "port_sweep.txt"
    ports = [{"impedance": 73.1 + 42.5j, "swr": 2.25}, {"impedance": 50.0 - 1e-5j, "swr": 1.0}]
    write_port_sweep(p, [300e6, 450e6], ports, 50.0)
    assert p.read_text().splitlines() == [
        "# Port sweep results, Z0 = 50.0 Ohm",
        "# step  frequency    Re(Z)    Im(Z)    SWR",
        "0 3e+08 73.1 42.5 2.25",
        "1 4.5e+08 50 -1e-05 1",
    ]


def test_radiation_diagram_and_rcs_layout(tmp_path):
    g = np.full(360, 1.5)
    g[0] = 1.0
    p = tmp_path / "polar_0.txt"
    write_radiation_diagrams(p, 3e8, g, g * 2, g * 10)
    lines = p.read_text().splitlines()
    assert lines[0] == "# FRICO radiation patterns. Frequency = 3e+08"
    assert lines[1] == "# angle XY_lin XY_dB YZ_lin YZ_dB XZ_lin XZ_dB"
    assert lines[2] == "0 1 0 2 3.010299956639812 10 10"
    assert len(lines) == 362
    r = np.arange(359 * 4, dtype=float).reshape(359, 4)
    q = tmp_path / "bistatic_rcs_0.txt"
    write_bistatic_rcs(q, r)
    lines = q.read_text().splitlines()
    assert lines[:2] == ["# FRICO bistatic RCS computation", "# Angle, VV_theta, HH_theta, VV_phi, HH_phi"]
    assert lines[3] == "1 4 5 6 7" and len(lines) == 361


def test_antenna_sweep_files(tmp_path):
    from frico_gb300.solver import AntennaResult
    g = np.ones(360)
    res = [AntennaResult(f, {"impedance": 70 + 1j * i, "swr": 1.5}, g, g, g) for i, f in enumerate([1e8, 2e8])]
    paths = write_antenna_sweep(tmp_path, res)
    assert [p.name for p in paths] == ["polar_0.txt", "polar_1.txt", "port_sweep.txt"]


@pytest.mark.parametrize("spec,axis", [("xy:1:2:0.1", (0, 0, 1)), ("yz:1:1:0.25", (0, 1, 0)),
                                       ("xz:0.5:0.5:0.1", (1, 0, 0)), ("0:0:2:1:1:0.5", (0, 0, 1))])
def test_sampling_plane_parse_and_grid(spec, axis):
    sp = parse_sampling_plane(spec)
    assert np.allclose(sp.normal, axis)
    P = sampling_plane_points(sp)
    # the xy rectangle is rotated about the axis by 90 degrees
    ext = np.ptp(P, axis=0)
    assert np.isclose(sorted(ext)[-1], max(sp.width, sp.height))
    if spec.startswith("xy"):
        assert np.allclose(P[:, 2], 0)
    if spec.startswith("yz"):
        assert np.allclose(P[:, 0], 0)
    if spec.startswith("xz"):
        assert np.allclose(P[:, 1], 0)


@pytest.mark.parametrize("spec", ["ab:1:1:0.1", "xy:1:1", "xy:a:1:0.1", "xy:1:1:0", "1:2:3:4:5"])
def test_sampling_plane_rejects(spec):
    with pytest.raises(ValueError):
        parse_sampling_plane(spec)
