"""GMSH ASCII mesh files (formats 4.1 and 2.2): the reader gives FRICO's view of
a mesh (src/input_gmsh.cpp:37-210: node order, triangles tagged by surface
entity, line elements tagged by curve entity, physical groups by name), and the
RWG table built from a file equals the one built from the same mesh in memory."""
import numpy as np
import pytest

from frico_gb300 import meshes

SMALL_41 = """$MeshFormat
4.1 0 8
$EndMeshFormat
$PhysicalNames
2
1 7 "feed"
2 8 "plate"
$EndPhysicalNames
$Entities
0 1 2 0
4 0 0 0 0 1 0 1 7 0
1 0 0 0 1 1 0 1 8 0
2 -1 0 0 0 1 0 1 8 0
$EndEntities
$Nodes
2 6 10 60
1 4 1 2
10
20
0 0 0 0
0 1 0 1
2 1 0 4
30
40
50
60
1 0 0
1 1 0
-1 0 0
-1 1 0
$EndNodes
$Elements
3 5 1 5
1 4 1 1
1 10 20
2 1 2 2
2 10 30 40
3 10 40 20
2 2 2 2
4 50 10 20
5 50 20 60
$EndElements
"""


def _arrays_equal(a, b):
    return all(np.array_equal(getattr(a, f), getattr(b, f)) for f in
               ("vertices", "triangles", "tri_tags", "curves", "curve_tags"))


@pytest.mark.parametrize("version", ["4.1", "2.2"])
@pytest.mark.parametrize("make", [meshes.strip_dipole, lambda: meshes.bowtie(8, 5), lambda: meshes.icosphere(2)])
def test_round_trip(tmp_path, version, make):
    m = make()
    m.physical = {"feed": (1, (meshes.FEED_TAG,))} if m.curves.shape[0] else {}
    f = tmp_path / f"m{version}.msh"
    meshes.write_msh(m, f, version)
    r = meshes.read_msh(f)
    assert _arrays_equal(r, m)
    assert r.physical == m.physical


def test_small_file_layout(tmp_path):
    """Two node blocks (one parametric), a line on curve 4, two surfaces."""
    f = tmp_path / "small.msh"
    f.write_text(SMALL_41)
    m = meshes.read_msh(f)
    np.testing.assert_array_equal(m.vertices[:, :2], [[0, 0], [0, 1], [1, 0], [1, 1], [-1, 0], [-1, 1]])
    np.testing.assert_array_equal(m.triangles, [[0, 2, 3], [0, 3, 1], [4, 0, 1], [4, 1, 5]])
    np.testing.assert_array_equal(m.tri_tags, [1, 1, 2, 2])
    np.testing.assert_array_equal(m.curves, [[0, 1]])
    np.testing.assert_array_equal(m.curve_tags, [4])
    assert m.physical == {"feed": (1, (4,)), "plate": (2, (1, 2))}
    assert m.entity_tags("feed") == (4,)
    # FRICO's skip list drops whole surfaces
    assert meshes.read_msh(f, skip_tags=[2]).nt == 2


def test_function_space_from_file(gpu_lib, tmp_path):
    """The RWG table (matrix order, T-/T+, feed interfaces) is the same whether the
    strip comes from memory or from a GMSH file; the file's feed is found by name."""
    from frico_gb300.solver import make_function_space
    m = meshes.strip_dipole()
    m.physical = {"feed": (1, (meshes.FEED_TAG,))}
    f = tmp_path / "strip.msh"
    meshes.write_msh(m, f)
    r = meshes.read_msh(f)
    a, b = make_function_space(m), make_function_space(r)
    assert a.n == b.n == 119
    for name in a.rwg.dtype.names:
        np.testing.assert_array_equal(a.rwg[name], b.rwg[name])
    assert r.entity_tags("feed") == (meshes.FEED_TAG,)


def test_rejects_unsupported(tmp_path):
    f = tmp_path / "bin.msh"
    f.write_text("$MeshFormat\n4.1 1 8\n$EndMeshFormat\n")
    with pytest.raises(ValueError, match="binary"):
        meshes.read_msh(f)
    f2 = tmp_path / "quad.msh"
    f2.write_text(SMALL_41.replace("2 1 2 2\n2 10 30 40\n3 10 40 20", "2 1 3 1\n2 10 30 40 20"))
    with pytest.raises(ValueError, match="element type 3"):
        meshes.read_msh(f2)
    f3 = tmp_path / "missing.msh"
    f3.write_text(SMALL_41.replace("1 10 20\n", "1 10 99\n"))
    with pytest.raises(ValueError, match="node 99"):
        meshes.read_msh(f3)
