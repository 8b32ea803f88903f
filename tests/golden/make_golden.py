"""Generate tests/golden/*.npz from FRICO's own sources compiled in place.

Run on a machine that has the FRICO checkout:
    make -C oracle/ref REF=<frico checkout>      # builds oracle/_ref/libfrico_ref.so
    python tests/golden/make_golden.py

Fixtures (all from FRICO's code, through oracle/ref/ref_driver.cpp):
  quadrature.npz  dunavant() points/weights, degrees 0..20, one triangle
  strip.npz       strip dipole: RWG table, Z (quadrature, degree 1), Z (-A),
                  delta-gap V, I, lumped currents, port values, E/H on a 10 deg
                  grid at R = 10 m, the three 360-point gain cuts
  sphere1.npz     level-1 icosphere: Z at degrees 2 and 5, plane-wave V, I,
                  bistatic 359-angle sigma table
  bowtie.npz      6 x 4 bowtie: RWG table, forced delta-gap orientation signs,
                  delta-gap V with those signs
  sphere4.npz     level-4 icosphere (N = 7680, the benchmarked size) at 450 MHz:
                  6 seeded columns of Z, the 2-norm of every column and the
                  Frobenius norm of Z, the plane-wave V and FRICO's solution I
                  (solve_general); with the oracle's term magnitudes of the sampled
                  columns (the tolerance scale where an entry's blocks cancel)
                  (`python tests/golden/make_golden.py sphere4`: about a minute)
  bowtie1500.npz  the N ~ 1500 bowtie of the sweep at 500 MHz, delta-gap feed with
                  FRICO's reorientation: 6 seeded columns of Z (with the oracle's
                  term magnitudes), V, FRICO's I and port values, and kappa_1(Z)
                  from LAPACK's zgecon (the scale of the solution's tolerance)
                  (`python tests/golden/make_golden.py bowtie1500`)
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

from frico_gb300 import meshes  # noqa: E402
import ref_frico  # noqa: E402

TRI = (np.array([0.1, 0.2, 0.3]), np.array([1.3, -0.2, 0.1]), np.array([0.4, 0.9, -0.5]))


def make_sphere4():
    from oracle import Oracle
    f = 450e6
    m = meshes.icosphere(4)
    r = ref_frico.RefFrico(m)
    Z = r.compute_matrix(f)
    cols = np.sort(np.random.default_rng(20261204).choice(r.n, 6, replace=False))
    V = r.rhs_plane_wave(f, 0.0, 0.0, 1.0, 0.0)
    I, _, _, _ = r.run_context_plane_wave(f, 0.0, 0.0, 1.0, 0.0)
    M = np.stack([Oracle(m).compute_matrix_magnitudes(f, int(c), int(c) + 1)[:, 0] for c in cols], axis=1)
    np.savez_compressed(HERE / "sphere4.npz", freq=f, cols=cols, Zcols=np.ascontiguousarray(Z[:, cols]),
                        Mcols=M, colnorms=np.linalg.norm(Z, axis=0), fro=np.linalg.norm(Z), V=V, I=I)
    print("sphere4.npz", (HERE / "sphere4.npz").stat().st_size)


def make_bowtie1500():
    from oracle import Oracle
    from scipy.linalg import lapack
    f = 500e6
    m = meshes.bowtie_preset(1500)
    r = ref_frico.RefFrico(m)
    signs = r.reorient([meshes.FEED_TAG])
    Z = r.compute_matrix(f)
    cols = np.sort(np.random.default_rng(20261205).choice(r.n, 6, replace=False))
    V = r.rhs_delta_gap(f, [meshes.FEED_TAG])
    I, _, _, _ = r.run_context_delta_gap(f, [meshes.FEED_TAG])
    pv = r.port_values([meshes.FEED_TAG])
    lu, _, _ = lapack.zgetrf(np.array(Z, order="F", copy=True))
    rcond, _ = lapack.zgecon(lu, np.abs(Z).sum(axis=0).max(), norm="1")
    M = np.stack([Oracle(m).compute_matrix_magnitudes(f, int(c), int(c) + 1)[:, 0] for c in cols], axis=1)
    np.savez_compressed(HERE / "bowtie1500.npz", freq=f, reoriented=signs is not None,
                        signs=signs if signs is not None else np.zeros(r.n),
                        cols=cols, Zcols=np.ascontiguousarray(Z[:, cols]), Mcols=M, V=V, I=I,
                        port=np.array([pv["current"], pv["power"], pv["impedance"], pv["gamma"], pv["swr"]]),
                        kappa1=1.0 / rcond)
    print("bowtie1500.npz", (HERE / "bowtie1500.npz").stat().st_size, "kappa_1 %.2e" % (1.0 / rcond))


def main():
    if not ref_frico.available():
        raise SystemExit("oracle/_ref/libfrico_ref.so missing: build it with oracle/ref/Makefile first")
    q = {f"deg{d}": ref_frico.dunavant(d, *TRI) for d in range(0, 21)}
    np.savez_compressed(HERE / "quadrature.npz", p0=TRI[0], p1=TRI[1], p2=TRI[2], **q)

    f = 300e6
    m = meshes.strip_dipole()
    r = ref_frico.RefFrico(m)
    Z = r.compute_matrix(f)
    Za = r.compute_matrix(f, approx=True)
    V = r.rhs_delta_gap(f, [meshes.FEED_TAG])
    I, AJ, AD, J = r.run_context_delta_gap(f, [meshes.FEED_TAG])
    pv = r.port_values([meshes.FEED_TAG])
    T, P, pts = meshes.far_field_grid(10.0, 10.0)
    E, H = r.eval_fields(pts)
    gains = np.stack([r.gain(pv["power"].real, 10.0, p) for p in range(3)])
    np.savez_compressed(HERE / "strip.npz", freq=f, rwg=r.rwg(), Z=Z, Z_approx=Za, V=V, I=I, AJ=AJ, AdivJ=AD, J=J,
                        port=np.array([pv["current"], pv["power"], pv["impedance"], pv["gamma"], pv["swr"]]),
                        points=pts, E=E, H=H, gains=gains)

    f = 450e6
    m = meshes.icosphere(1)
    out = {"freq": f}
    for d in (2, 5):
        r = ref_frico.RefFrico(m, degree=d)
        out[f"Z_deg{d}"] = r.compute_matrix(f)
    r = ref_frico.RefFrico(m)
    out["V"] = r.rhs_plane_wave(f, 0.0, 0.0, 1.0, 0.0)
    out["I"], out["AJ"], out["AdivJ"], out["J"] = r.run_context_plane_wave(f, 0.0, 0.0, 1.0, 0.0)
    out["bistatic"] = r.bistatic_rcs(10.0)
    np.savez_compressed(HERE / "sphere1.npz", **out)

    m = meshes.bowtie(6, 4)
    r = ref_frico.RefFrico(m)
    signs = r.reorient([meshes.FEED_TAG], force=True)
    # delta-gap V with those signs (update_rhs reads sim.delta_gap_signs)
    V = r.rhs_delta_gap(500e6, [meshes.FEED_TAG])
    np.savez_compressed(HERE / "bowtie.npz", rwg=r.rwg(), signs=signs, V=V, freq=500e6)
    for p in sorted(HERE.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    if sys.argv[1:] in (["sphere4"], ["bowtie1500"]):
        if not ref_frico.available():
            raise SystemExit("oracle/_ref/libfrico_ref.so missing: build it with oracle/ref/Makefile first")
        make_sphere4() if sys.argv[1] == "sphere4" else make_bowtie1500()
    else:
        main()
