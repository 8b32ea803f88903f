"""CPU tests: synthetic meshes, host-side mesh front end, ABI exports, oracle sanity."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from frico_gb300 import meshes

ROOT = Path(__file__).resolve().parent.parent


def test_mesh_sizes():
    s = meshes.strip_dipole()
    assert (s.nt, s.nv) == (120, 122)
    for lvl, nt in ((1, 80), (2, 320), (4, 5120), (5, 20480)):
        m = meshes.icosphere(lvl, jitter=0.0 if lvl == 5 else 0.03)
        assert m.nt == nt
    r = np.linalg.norm(meshes.icosphere(3).vertices, axis=1)
    assert np.allclose(r, 1.0, atol=1e-14)


def test_icosphere_seeded():
    a = meshes.icosphere(2)
    b = meshes.icosphere(2)
    assert np.array_equal(a.vertices, b.vertices)
    c = meshes.icosphere(2, jitter=0.0)
    d = np.linalg.norm(a.vertices - c.vertices, axis=1)
    assert 0 < d.max() < 0.03 * 0.5  # within 3% of the local edge length (~0.27 at level 2... bound loosely)


def test_function_space_matches_oracle(gpu_lib):
    from frico_gb300.solver import make_function_space
    from oracle import Oracle
    for mesh in (meshes.strip_dipole(), meshes.icosphere(2), meshes.bowtie(6, 4)):
        fs = make_function_space(mesh)
        o = Oracle(mesh)
        r = o.rwg()
        assert fs.n == o.n
        rw = fs.rwg
        assert np.array_equal(rw["Aminus"], r[:, 0]) and np.array_equal(rw["Aplus"], r[:, 1])
        assert np.array_equal(rw["itminus"], r[:, 2].astype(np.int64))
        assert np.array_equal(rw["itplus"], r[:, 3].astype(np.int64))
        assert np.array_equal(rw["pminus"], r[:, 4:7]) and np.array_equal(rw["pplus"], r[:, 7:10])
        assert np.array_equal(rw["length"], r[:, 10])
        assert np.array_equal(rw["edge_index"], r[:, 11].astype(np.int64))
        assert np.array_equal(rw["matrix_index"], np.arange(fs.n))
        assert np.array_equal(rw["has_interface"], r[:, 13].astype(np.int32))
        assert np.array_equal(fs.edge_vertices, r[:, 15:17].astype(np.int64))
        assert np.all(rw["itminus"] < rw["itplus"])


def test_rwg_counts(gpu_lib):
    from frico_gb300.solver import make_function_space
    assert make_function_space(meshes.strip_dipole()).n == 119
    assert make_function_space(meshes.icosphere(4)).n == 7680
    for target, (nx, ny) in meshes.BOWTIE_PRESETS.items():
        n = make_function_space(meshes.bowtie(nx, ny)).n
        assert n == 6 * nx * ny - 2 * nx - ny
        assert abs(n - target) / target < 0.06


def test_feed_interfaces(gpu_lib):
    from frico_gb300.solver import make_function_space
    fs = make_function_space(meshes.strip_dipole())
    feed = np.nonzero(fs.rwg["has_interface"])[0]
    assert len(feed) == 1 and fs.rwg["interface_tag"][feed[0]] == meshes.FEED_TAG
    fs = make_function_space(meshes.bowtie(8, 5))
    assert int(fs.rwg["has_interface"].sum()) == 5


def test_reorient_matches_oracle(gpu_lib):
    from frico_gb300.solver import make_function_space, reorient_deltagap_edges
    from oracle import Oracle
    m = meshes.bowtie(8, 5)
    fs = make_function_space(m)
    o = Oracle(m)
    assert reorient_deltagap_edges(fs, [meshes.FEED_TAG]) is None   # arm 1 numbered first
    assert o.reorient([meshes.FEED_TAG]) is None
    s1 = reorient_deltagap_edges(fs, [meshes.FEED_TAG], force=True)
    s2 = o.reorient([meshes.FEED_TAG], force=True)
    assert np.array_equal(s1, s2)
    # swapped surface tags trigger the reorientation
    m2 = meshes.bowtie(8, 5)
    m2.tri_tags = 3 - m2.tri_tags
    fs2 = make_function_space(m2)
    o2 = Oracle(m2)
    a, b = reorient_deltagap_edges(fs2, [meshes.FEED_TAG]), o2.reorient([meshes.FEED_TAG])
    assert a is not None and np.array_equal(a, b)


def test_mesh_errors(gpu_lib):
    from frico_gb300 import FricoError
    from frico_gb300.solver import make_function_space
    m = meshes.strip_dipole()
    bad = meshes.TriMesh("lonely", m.vertices, m.triangles, m.tri_tags, np.array([[0, 5]]), np.array([9], np.int32))
    with pytest.raises(FricoError) as e:
        make_function_space(bad)
    assert e.value.code == -8
    T = np.concatenate([m.triangles, m.triangles[:1]])
    with pytest.raises(FricoError):
        make_function_space(meshes.TriMesh("dup", m.vertices, T, np.ones(len(T), np.int32)))


def test_abi_exports_every_declared_symbol(gpu_lib):
    header = (ROOT / "include" / "frico_gpu.h").read_text()
    names = set(re.findall(r"\b(frico_gpu_\w+)\s*\(", header))
    assert len(names) >= 20
    lib = ctypes.CDLL(str(ROOT / "frico_gb300" / "_lib" / "libfrico_gpu.so"))
    for nm in sorted(names):
        assert hasattr(lib, nm), nm


def test_abi_constants_match_header():
    """Every integer constant the Python binding mirrors has the header's value."""
    from frico_gb300 import _abi
    header = (ROOT / "include" / "frico_gpu.h").read_text()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+FRICO_(\w+)\s+(-?\d+)\b", header)}
    mirrored = 0
    for name, value in defs.items():
        key = name[len("GPU_"):] if name.startswith("GPU_") else name
        if hasattr(_abi, key):
            assert getattr(_abi, key) == value, name
            mirrored += 1
    for group in ("GEMM_", "PIVOT_", "REFINE_", "RESIDUAL_", "PREC_", "HPHASE_", "EDGE_LENGTH_"):
        names = [n for n in defs if n.startswith(group)]
        assert names and all(hasattr(_abi, n) for n in names), group
    assert mirrored >= 25


def test_build_can_be_called_again_in_one_process(gpu_lib):
    import frico_gb300
    frico_gb300.build()
    frico_gb300.build()
    assert callable(frico_gb300.build)


def test_ctx_create_without_gpu_fails_cleanly(gpu_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    ctx = ctypes.c_void_p()
    assert gpu_lib.frico_gpu_ctx_create(ctypes.byref(ctx), 0, None) == -5


def test_oracle_physics_strip():
    from oracle import Oracle
    m = meshes.strip_dipole()
    o = Oracle(m)
    Z = o.compute_matrix(300e6)
    I = o.solve(Z, o.rhs_delta_gap(300e6, [meshes.FEED_TAG]))
    pv = o.port_values(I, o.rwg(), [meshes.FEED_TAG])
    assert 65 < pv["impedance"].real < 85 and abs(pv["impedance"].imag) < 30
    o.lump(300e6, I)
    G = o.gain(pv["power"].real, 10.0, 1)
    assert 1.9 < 10 * np.log10(G.max()) < 2.4        # dipole: ~2.15 dB
    Za = o.compute_matrix(300e6, approx=True)
    # MOM3D Z is symmetric up to the summation order of the -+ / +- blocks
    assert np.abs(Za - Za.T).max() < 1e-14 * np.abs(Za).max()
    # the split rule breaks symmetry at the quadrature-error level
    assert np.abs(Z - Z.T).max() > 1e-6 * np.abs(Z).max()


def test_oracle_dunavant_exactness():
    """Each Dunavant rule integrates monomials up to its degree; weights sum to the area."""
    from oracle import dunavant
    p0, p1, p2 = np.array([0.0, 0.0, 0.0]), np.array([1.0, 0.0, 0.0]), np.array([0.0, 1.0, 0.0])
    for d in range(1, 21):
        q = dunavant(d, p0, p1, p2)
        assert abs(q[:, 3].sum() - 0.5) < 1e-12
        for a in range(d + 1):
            b = d - a
            exact = np.math.factorial(a) * np.math.factorial(b) / np.math.factorial(a + b + 2) \
                if hasattr(np, "math") else None
            if exact is None:
                import math
                exact = math.factorial(a) * math.factorial(b) / math.factorial(a + b + 2)
            got = np.sum(q[:, 3] * q[:, 0] ** a * q[:, 1] ** b)
            assert abs(got - exact) < 1e-11, (d, a, b, got, exact)


def test_abi_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of the C-ABI's structs have the sizes and field offsets
    the C compiler gives the header's declarations."""
    import shutil
    import subprocess
    from frico_gb300 import _abi
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    structs = {"frico_gpu_options": _abi.Options, "frico_gpu_stats": _abi.Stats,
               "frico_sweep_report": _abi.SweepReport, "frico_adjoint_result": _abi.AdjointResult,
               "frico_port_values": _abi.PortValues}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "frico_gpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
