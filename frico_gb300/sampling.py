"""Near-field sampling planes (FRICO's -p option): parse_sampling_plane and
make_sampling_plane_mesh (src/sampling_planes.cpp:42-157), evaluated by
write_fields' per-vertex eval_fields loop (src/emw_postpro_common.cpp:161-201).

FRICO meshes the rectangle [-w/2, w/2] x [-h/2, h/2] (z = 0) with GMSH at
element size `size`, then rotates it by pi/2 about the axis `normal` (which is
how "yz" / "xz" planes come out of the xy rectangle). GMSH is not available
here, so the rectangle gets a structured grid of spacing <= size; the fields
are evaluated on the GPU (frico_gpu_eval_fields) at its vertices. SILO output
is replaced by a text file (x y z, then Re/Im of E and H).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class SamplingPlane:
    width: float
    height: float
    size: float
    normal: np.ndarray   # rotation axis (unit vector)


def parse_sampling_plane(spec: str) -> SamplingPlane:
    """'xy|yz|xz:width:height:size' or 'nx:ny:nz:width:height:size'. The short
    forms map to the axes FRICO uses: xy -> z, yz -> y, xz -> x."""
    toks = spec.split(":")
    try:
        if len(toks) == 4:
            axis = {"xy": (0.0, 0.0, 1.0), "yz": (0.0, 1.0, 0.0), "xz": (1.0, 0.0, 0.0)}.get(toks[0])
            if axis is None:
                raise ValueError(f"unknown plane '{toks[0]}'")
            n = np.array(axis)
            w, h, s = float(toks[1]), float(toks[2]), float(toks[3])
        elif len(toks) == 6:
            n = np.array([float(toks[0]), float(toks[1]), float(toks[2])])
            n = n / np.linalg.norm(n)
            w, h, s = float(toks[3]), float(toks[4]), float(toks[5])
        else:
            raise ValueError("expected 4 or 6 ':'-separated fields")
    except ValueError as e:
        raise ValueError(f"bad sampling plane '{spec}': {e}") from None
    if not (w > 0 and h > 0 and s > 0):
        raise ValueError(f"bad sampling plane '{spec}': sizes must be > 0")
    return SamplingPlane(w, h, s, n)


def _rotation(axis: np.ndarray, angle: float) -> np.ndarray:
    """Rodrigues rotation matrix about a unit axis."""
    x, y, z = axis
    c, s = np.cos(angle), np.sin(angle)
    K = np.array([[0, -z, y], [z, 0, -x], [-y, x, 0]])
    return np.eye(3) + s * K + (1 - c) * (K @ K)


def sampling_plane_points(sp: SamplingPlane) -> np.ndarray:
    """Vertices of the plane's grid, (npts, 3)."""
    nx = max(1, int(np.ceil(sp.width / sp.size - 1e-12)))
    ny = max(1, int(np.ceil(sp.height / sp.size - 1e-12)))
    xs = np.linspace(-sp.width / 2, sp.width / 2, nx + 1)
    ys = np.linspace(-sp.height / 2, sp.height / 2, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    P = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)
    return P @ _rotation(sp.normal, np.pi / 2).T


def sample_plane(sim, spec: str, col: int = 0):
    """(points, E, H) on a sampling plane for RHS column `col` of a solved simulation."""
    P = sampling_plane_points(parse_sampling_plane(spec))
    E, H = sim.eval_fields(P, col=col)
    return P, E, H


def write_sampling_plane(path, P, E, H) -> None:
    """One line per vertex: x y z Re(Ex) Im(Ex) ... Re(Hz) Im(Hz)."""
    from .outputs import cpp_format
    with open(path, "w") as f:
        f.write("# FRICO sampling plane: x y z Ex Ey Ez Hx Hy Hz (re im)\n")
        for p, e, h in zip(P, E, H):
            vals = list(p) + [v for z in list(e) + list(h) for v in (z.real, z.imag)]
            f.write(" ".join(cpp_format(v) for v in vals) + "\n")
