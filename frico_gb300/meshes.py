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
"""
from __future__ import annotations

from dataclasses import dataclass, field

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
