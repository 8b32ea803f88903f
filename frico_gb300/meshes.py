"""Seeded synthetic meshes and observation grids.

FRICO reads GMSH meshes; GMSH is not available here, so the workloads are
built as triangle soups with the same ingredients a GMSH model hands to
load_from_gmsh (src/input_gmsh.cpp:324-406): vertex coordinates, triangles
tagged by surface, and tagged 1-D curve segments (the delta-gap feed).

  strip_dipole   0.48 m x 5 mm strip in z = 0, 60 x 1 rectangles split on one
                 diagonal: 120 triangles, 119 RWG edges, feed = centre
                 transverse edge (curve tag 3); left half tag 1, right tag 2.
  icosphere      icosahedron subdivided `level` times, projected to radius R,
                 tangential jitter uniform in +-3% of the local mean edge
                 length, re-projected (level 4: 5120 tri / 7680 RWG;
                 level 5: 20480 / 30720).
  bowtie         two isosceles arms along -x / +x, arm length 0.25 m, flare
                 60 deg, joined by a 5 mm feed column of collinear edges
                 (curve tag 3); arm 1 tag 1 numbered first, arm 2 tag 2;
                 interior vertices jittered by +-10% of the local cell size.

Meshes made by GMSH itself are read from its ASCII files (read_msh, formats
4.1 and 2.2) and synthetic ones written out (write_msh) for GMSH or FRICO.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

FEED_TAG = 3


@dataclass
class TriMesh:
    name: str
    vertices: np.ndarray          # (nv, 3) float64
    triangles: np.ndarray         # (nt, 3) int64
    tri_tags: np.ndarray          # (nt,) int32
    curves: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int64))
    curve_tags: np.ndarray = field(default_factory=lambda: np.zeros((0,), np.int32))
    feed_tags: tuple = ()
    # physical groups by name: (dimension, entity tags), as FRICO looks a feed up by name
    physical: dict = field(default_factory=dict)

    def entity_tags(self, name: str) -> tuple:
        """Entity tags of a physical group (e.g. the curves of a delta-gap feed)."""
        return tuple(self.physical[name][1])

    @property
    def nv(self) -> int:
        return int(self.vertices.shape[0])

    @property
    def nt(self) -> int:
        return int(self.triangles.shape[0])


def strip_dipole(length: float = 0.48, width: float = 0.005, nx: int = 60) -> TriMesh:
    i = np.arange(nx + 1)
    xs = -length / 2 + i * (length / nx)
    verts = np.zeros((2 * (nx + 1), 3))
    verts[0::2, 0] = xs
    verts[1::2, 0] = xs
    verts[0::2, 1] = -width / 2
    verts[1::2, 1] = width / 2

    def v(ii, j):
        return 2 * ii + j

    tris, tags = [], []
    for ii in range(nx):
        tag = 1 if ii < nx // 2 else 2
        tris.append((v(ii, 0), v(ii + 1, 0), v(ii + 1, 1)))
        tris.append((v(ii, 0), v(ii + 1, 1), v(ii, 1)))
        tags += [tag, tag]
    c = nx // 2
    return TriMesh("strip", verts, np.array(tris, np.int64), np.array(tags, np.int32),
                   np.array([[v(c, 0), v(c, 1)]], np.int64), np.array([FEED_TAG], np.int32),
                   (FEED_TAG,))


def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], float)
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
         (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
         (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
         (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return [tuple(x) for x in v], f


def icosphere(level: int, radius: float = 1.0, jitter: float = 0.03,
              seed: int = 20260101) -> TriMesh:
    verts, faces = _icosahedron()
    verts = [np.array(p) for p in verts]
    for _ in range(level):
        cache: dict = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    V = np.array(verts) * radius
    F = np.array(faces, np.int64)
    if jitter > 0:
        nv = V.shape[0]
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
        e = np.unique(np.sort(e, axis=1), axis=0)
        L = np.linalg.norm(V[e[:, 0]] - V[e[:, 1]], axis=1)
        acc = np.zeros(nv)
        cnt = np.zeros(nv)
        np.add.at(acc, e[:, 0], L)
        np.add.at(acc, e[:, 1], L)
        np.add.at(cnt, e[:, 0], 1)
        np.add.at(cnt, e[:, 1], 1)
        h = acc / cnt
        n = V / np.linalg.norm(V, axis=1, keepdims=True)
        ref = np.where(np.abs(n[:, 2:3]) < 0.9, np.array([[0.0, 0.0, 1.0]]), np.array([[1.0, 0.0, 0.0]]))
        e1 = np.cross(n, ref)
        e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
        e2 = np.cross(n, e1)
        u = np.random.default_rng(seed).uniform(-1.0, 1.0, size=(nv, 2))
        V = V + (jitter * h)[:, None] * (u[:, 0:1] * e1 + u[:, 1:2] * e2)
        V = radius * V / np.linalg.norm(V, axis=1, keepdims=True)
    return TriMesh(f"icosphere{level}", V, F, np.ones(F.shape[0], np.int32))


BOWTIE_PRESETS = {500: (13, 7), 1500: (22, 12), 3000: (30, 17)}


def bowtie(nx: int, ny: int, arm: float = 0.25, flare_deg: float = 60.0, gap: float = 0.005,
           jitter: float = 0.10, seed: int = 20260102) -> TriMesh:
    tan_h = np.tan(np.radians(flare_deg) / 2)
    rng = np.random.default_rng(seed)
    nper = (nx + 1) * (ny + 1)
    verts = np.zeros((nper + nx * (ny + 1), 3))

    def vid(a, ix, iy):
        if a == 1 or ix == nx:
            return ix * (ny + 1) + iy
        return nper + ix * (ny + 1) + iy

    for a in (1, 2):
        for ix in range(nx + 1):
            if a == 2 and ix == nx:
                continue
            d = arm - arm * ix / nx                 # distance from the feed
            x = -d if a == 1 else d
            w = gap / 2 + d * tan_h
            for iy in range(ny + 1):
                y = -w + 2 * w * iy / ny
                dx = dy = 0.0
                if 0 < ix < nx and 0 < iy < ny and jitter > 0:
                    u = rng.uniform(-1.0, 1.0, 2)
                    dx = jitter * u[0] * arm / nx
                    dy = jitter * u[1] * 2 * w / ny
                verts[vid(a, ix, iy)] = (x + dx, y + dy, 0.0)
    tris, tags = [], []
    for a in (1, 2):
        for ix in range(nx):
            for iy in range(ny):
                v00, v10 = vid(a, ix, iy), vid(a, ix + 1, iy)
                v11, v01 = vid(a, ix + 1, iy + 1), vid(a, ix, iy + 1)
                if a == 1:
                    tris += [(v00, v10, v11), (v00, v11, v01)]
                else:
                    tris += [(v00, v11, v10), (v00, v01, v11)]
                tags += [a, a]
    feed = [(vid(1, nx, iy), vid(1, nx, iy + 1)) for iy in range(ny)]
    return TriMesh(f"bowtie{nx}x{ny}", verts, np.array(tris, np.int64), np.array(tags, np.int32),
                   np.array(feed, np.int64), np.full(len(feed), FEED_TAG, np.int32), (FEED_TAG,))


def bowtie_flare_tangent(nx: int, ny: int, flare_deg: float = 60.0, **kw) -> np.ndarray:
    """d(vertices)/d(flare angle in radians) of bowtie(nx, ny, flare_deg=...): the
    vertices depend on the flare only through tan(flare/2), linearly, so a
    central difference in the angle (h = 1e-6 rad) is accurate to ~1e-9."""
    h = 1e-6
    hd = np.degrees(h)
    vp = bowtie(nx, ny, flare_deg=flare_deg + hd, **kw).vertices
    vm = bowtie(nx, ny, flare_deg=flare_deg - hd, **kw).vertices
    return (vp - vm) / (2 * h)


def bowtie_preset(n_target: int, **kw) -> TriMesh:
    nx, ny = BOWTIE_PRESETS[n_target]
    return bowtie(nx, ny, **kw)


def sweep_frequencies(f0: float = 200e6, f1: float = 800e6, count: int = 256) -> np.ndarray:
    """f_i = f0 + i (f1 - f0)/(count - 1), computed directly (no accumulation)."""
    i = np.arange(count, dtype=np.float64)
    return f0 + i * (f1 - f0) / (count - 1)


def sph2rect(R: float, theta, phi) -> np.ndarray:
    """src/utils.h:54-61."""
    theta = np.asarray(theta, float)
    phi = np.asarray(phi, float)
    return np.stack([R * np.cos(phi) * np.sin(theta), R * np.sin(phi) * np.sin(theta),
                     R * np.cos(theta) * np.ones_like(phi)], axis=-1)


def far_field_grid(R: float = 10.0, step_deg: float = 1.0):
    """theta in [0, 180] x phi in [0, 360) at `step_deg`; returns (theta, phi, points)."""
    th = np.radians(np.arange(0.0, 180.0 + 1e-9, step_deg))
    ph = np.radians(np.arange(0.0, 360.0 - 1e-9, step_deg))
    T, P = np.meshgrid(th, ph, indexing="ij")
    T, P = T.ravel(), P.ravel()
    return T, P, sph2rect(R, T, P)


def bistatic_cuts(R: float = 10.0, phis_deg=(0.0, 90.0)):
    """181 theta values (0..180 deg) on each of the given phi cuts."""
    th = np.radians(np.arange(0.0, 181.0))
    T = np.concatenate([th for _ in phis_deg])
    P = np.concatenate([np.full(th.shape, np.radians(p)) for p in phis_deg])
    return T, P, sph2rect(R, T, P)


# ------------------------------------------------------------------ GMSH files
_MSH_TRIANGLE, _MSH_LINE, _MSH_POINT = 2, 1, 15


def _msh_sections(text: str) -> dict:
    sections, name, body = {}, None, []
    for line in text.splitlines():
        t = line.strip()
        if t.startswith("$"):
            if t.startswith("$End"):
                sections.setdefault(name, body)
                name, body = None, []
            else:
                name, body = t[1:], []
        elif name is not None:
            body.append(t)
    return sections


def _msh_physical_names(sec: dict) -> dict:
    names = {}
    lines = sec.get("PhysicalNames", [])
    for line in lines[1:1 + int(lines[0])] if lines else []:
        dim, tag, rest = line.split(maxsplit=2)
        names[(int(dim), int(tag))] = rest.strip().strip('"')
    return names


def read_msh(path, skip_tags=(), name: str | None = None) -> TriMesh:
    """A GMSH ASCII mesh file (format 4.1 or 2.2) as FRICO's load_from_gmsh takes
    a mesh from the gmsh API (src/input_gmsh.cpp:37-210): the vertices in the
    file's node order, the 3-node triangles of every surface entity whose tag is
    not in skip_tags, each tagged with its surface's entity tag, and the 2-node
    line elements tagged with their curve's entity tag (the interface tags of the
    RWG edges they lie on). Physical groups map their names to entity tags, as a
    delta-gap feed is named on FRICO's command line. Binary files and other
    element types (quadrangles, second-order elements) raise ValueError."""
    text = Path(path).read_text()
    sec = _msh_sections(text)
    if "MeshFormat" not in sec:
        raise ValueError(f"{path}: not a GMSH mesh file")
    fmt = sec["MeshFormat"][0].split()
    version, ftype = fmt[0], int(fmt[1])
    if ftype != 0:
        raise ValueError(f"{path}: binary GMSH files are not supported (write ASCII)")
    names = _msh_physical_names(sec)
    node_tags, coords = [], []
    tris, tri_tags, lines, line_tags = [], [], [], []
    phys_entities: dict = {}   # (dim, physical tag) -> set of entity tags
    skip = {int(t) for t in skip_tags}

    def element(dim, etype, ent, nodes, where):
        if etype == _MSH_TRIANGLE and dim == 2:
            if ent not in skip:
                tris.append(nodes[:3])
                tri_tags.append(ent)
        elif etype == _MSH_LINE and dim == 1:
            lines.append(nodes[:2])
            line_tags.append(ent)
        elif etype != _MSH_POINT:
            raise ValueError(f"{path}: element type {etype} on {where} is not supported "
                             "(3-node triangles and 2-node lines only)")

    if version.startswith("4"):
        ent = sec.get("Entities", [])
        if ent:
            counts = [int(x) for x in ent[0].split()]
            k = 1
            for dim in range(4):
                for _ in range(counts[dim]):
                    f = ent[k].split()
                    k += 1
                    tag = int(f[0])
                    np_at = 4 if dim == 0 else 7
                    for ph in f[np_at + 1: np_at + 1 + int(f[np_at])]:
                        phys_entities.setdefault((dim, abs(int(ph))), set()).add(tag)
        nod = sec["Nodes"]
        nblocks = int(nod[0].split()[0])
        k = 1
        for _ in range(nblocks):
            _, _, parametric, cnt = (int(x) for x in nod[k].split())
            k += 1
            node_tags.extend(int(nod[k + i]) for i in range(cnt))
            coords.extend([float(v) for v in nod[k + cnt + i].split()[:3]] for i in range(cnt))
            k += 2 * cnt
        el = sec["Elements"]
        nblocks = int(el[0].split()[0])
        k = 1
        for _ in range(nblocks):
            dim, etag, etype, cnt = (int(x) for x in el[k].split())
            k += 1
            for i in range(cnt):
                f = [int(x) for x in el[k + i].split()]
                element(dim, etype, etag, f[1:], f"entity ({dim}, {etag})")
            k += cnt
    elif version.startswith("2"):
        nod = sec["Nodes"]
        for line in nod[1:1 + int(nod[0])]:
            f = line.split()
            node_tags.append(int(f[0]))
            coords.append([float(v) for v in f[1:4]])
        el = sec["Elements"]
        dims = {_MSH_TRIANGLE: 2, _MSH_LINE: 1, _MSH_POINT: 0}
        for line in el[1:1 + int(el[0])]:
            f = [int(x) for x in line.split()]
            etype, ntags = f[1], f[2]
            tags, nodes = f[3:3 + ntags], f[3 + ntags:]
            phys = tags[0] if ntags > 0 else 0
            etag = tags[1] if ntags > 1 else phys   # elementary (entity) tag
            dim = dims.get(etype, -1)
            if phys and dim >= 0:
                phys_entities.setdefault((dim, phys), set()).add(etag)
            element(dim, etype, etag, nodes, f"element {f[0]}")
    else:
        raise ValueError(f"{path}: GMSH format {version} is not supported (4.1 or 2.2)")

    index = {t: i for i, t in enumerate(node_tags)}
    try:
        T = np.array([[index[v] for v in t] for t in tris], np.int64).reshape(-1, 3)
        Cv = np.array([[index[v] for v in c] for c in lines], np.int64).reshape(-1, 2)
    except KeyError as e:
        raise ValueError(f"{path}: element refers to node {e.args[0]}, which the file does not define") from None
    physical = {}
    for (dim, ph), ents in sorted(phys_entities.items()):
        physical[names.get((dim, ph), str(ph))] = (dim, tuple(sorted(ents)))
    return TriMesh(name or Path(path).stem, np.array(coords, np.float64).reshape(-1, 3), T,
                   np.array(tri_tags, np.int32), Cv, np.array(line_tags, np.int32), (), physical)


def write_msh(mesh: TriMesh, path, version: str = "4.1") -> None:
    """Write a mesh as a GMSH ASCII file (4.1 or 2.2): the triangles in blocks by
    surface tag, the tagged curve segments by curve tag, the vertices in order
    (tags 1..nv), and the physical groups by name. Coordinates are written with
    17 significant digits, so read_msh gives back the same arrays."""
    V, T, Cv = mesh.vertices, mesh.triangles, mesh.curves
    stags = sorted(set(int(t) for t in mesh.tri_tags))
    ctags = sorted(set(int(t) for t in mesh.curve_tags))
    groups = list(mesh.physical.items())
    phys_of: dict = {}   # (dim, entity tag) -> physical tags
    for k, (_, (dim, ents)) in enumerate(groups):
        for e in ents:
            phys_of.setdefault((dim, int(e)), []).append(k + 1)
    g = "{:.17g}".format
    out = ["$MeshFormat", f"{version} 0 8", "$EndMeshFormat"]
    if groups:
        out += ["$PhysicalNames", str(len(groups))]
        out += [f'{dim} {k + 1} "{nm}"' for k, (nm, (dim, _)) in enumerate(groups)]
        out += ["$EndPhysicalNames"]
    if version == "4.1":
        def box(idx):
            P = V[np.unique(idx)]
            return " ".join(g(x) for x in (*P.min(axis=0), *P.max(axis=0)))

        def entity(dim, tag, idx):
            ph = phys_of.get((dim, tag), [])
            return f"{tag} {box(idx)} {len(ph)}" + "".join(f" {p}" for p in ph) + " 0"

        out += ["$Entities", f"0 {len(ctags)} {len(stags)} 0"]
        out += [entity(1, t, Cv[mesh.curve_tags == t]) for t in ctags]
        out += [entity(2, t, T[mesh.tri_tags == t]) for t in stags]
        out += ["$EndEntities", "$Nodes", f"1 {len(V)} 1 {len(V)}", f"2 {stags[0]} 0 {len(V)}"]
        out += [str(i + 1) for i in range(len(V))]
        out += [" ".join(g(x) for x in v) for v in V]
        out += ["$EndNodes", "$Elements", f"{len(ctags) + len(stags)} {len(Cv) + len(T)} 1 {len(Cv) + len(T)}"]
        e = 0
        for t in ctags:
            sel = Cv[mesh.curve_tags == t]
            out.append(f"1 {t} {_MSH_LINE} {len(sel)}")
            for c in sel:
                e += 1
                out.append(f"{e} {c[0] + 1} {c[1] + 1}")
        for t in stags:
            sel = T[mesh.tri_tags == t]
            out.append(f"2 {t} {_MSH_TRIANGLE} {len(sel)}")
            for tri in sel:
                e += 1
                out.append(f"{e} {tri[0] + 1} {tri[1] + 1} {tri[2] + 1}")
        out += ["$EndElements"]
    elif version == "2.2":
        out += ["$Nodes", str(len(V))]
        out += [f"{i + 1} " + " ".join(g(x) for x in v) for i, v in enumerate(V)]
        out += ["$EndNodes", "$Elements", str(len(Cv) + len(T))]
        e = 0
        for dim, etype, sel, tags in ((1, _MSH_LINE, Cv, mesh.curve_tags), (2, _MSH_TRIANGLE, T, mesh.tri_tags)):
            for nodes, t in zip(sel, tags):
                e += 1
                ph = phys_of.get((dim, int(t)), [0])[0]
                out.append(f"{e} {etype} 2 {ph} {int(t)} " + " ".join(str(int(v) + 1) for v in nodes))
        out += ["$EndElements"]
    else:
        raise ValueError(f"GMSH format {version} is not written (4.1 or 2.2)")
    Path(path).write_text("\n".join(out) + "\n")
