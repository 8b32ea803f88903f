"""Post-processing beyond FRICO's default outputs, against the oracle:
monostatic RCS from one multi-RHS solve, and near-field sampling planes."""
import numpy as np
import pytest

from frico_gb300 import meshes
from frico_gb300.sampling import sample_plane
from frico_gb300.solver import DeltaGap, Simulation

DEG = np.pi / 180


def _rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.mark.gpu
def test_monostatic_rcs_matches_oracle(gpu_lib):
    from oracle import Oracle
    m = meshes.icosphere(2)
    f, R = 450e6, 10.0
    th = np.array([0.0, 60.0, 125.0]) * DEG
    ph = np.array([0.0, 30.0, 90.0]) * DEG
    sim = Simulation(m, precision="fp64")
    sig = sim.monostatic_rcs(f, th, ph, 1.0, 1.0, R)
    assert sig.shape == (3, 2)
    o = Oracle(m)
    Z = o.compute_matrix(f)
    for c in range(3):
        I = o.solve(Z, o.rhs_plane_wave(f, th[c], ph[c], 1.0, 1.0))
        o.lump(f, I)
        ref = o.rcs(R, [th[c]], [ph[c]])[0]
        assert _rel(sig[c], ref) < 1e-9


@pytest.mark.gpu
def test_sampling_plane_fields_match_oracle(gpu_lib):
    from oracle import Oracle
    m = meshes.strip_dipole()
    f = 300e6
    sim = Simulation(m, precision="fp64")
    I = sim.run_context(f, DeltaGap((meshes.FEED_TAG,), 1.0), download=True)
    P, E, H = sample_plane(sim, "xz:0.8:0.4:0.05")
    assert np.allclose(P[:, 1], 0.0) and P.shape[0] == 17 * 9
    o = Oracle(m)
    o.lump(f, I[:, 0])
    Er, Hr = o.eval_fields(P)
    assert _rel(E, Er) < 1e-9 and _rel(H, Hr) < 1e-9


@pytest.mark.gpu
def test_fields_multi_match_single_column(gpu_lib):
    from frico_gb300.solver import PlaneWave
    m = meshes.icosphere(2)
    f = 450e6
    sim = Simulation(m, precision="mixed")
    sim.compute_matrix(f)
    ncols = 7                                   # two column tiles, the second partial
    sim.set_nrhs(ncols)
    for c in range(ncols):
        sim.update_rhs(f, PlaneWave(c * 25 * DEG, c * 40 * DEG, 1.0, 0.5), c)
    sim.solve(download=False)
    th = np.linspace(0, np.pi, 37)
    ph = np.full(37, 0.7)
    P = meshes.sph2rect(10.0, th, ph)
    E, H = sim.eval_fields_multi(P)
    sig = sim.rcs_points_multi(10.0, th, ph)
    assert E.shape == (ncols, 37, 3) and sig.shape == (ncols, 37, 2)
    for c in range(ncols):
        # mixed precision: the single-column pass sums in double-float (about 2^-47
        # per operation), the multi-column pass in FP64
        Ec, Hc = sim.eval_fields(P, col=c)
        assert _rel(E[c], Ec) < 1e-11 and _rel(H[c], Hc) < 1e-11
        assert _rel(sig[c], sim.rcs_points(10.0, th, ph, col=c)) < 1e-11
    E2, H2 = sim.eval_fields_multi(P, col0=2, ncols=3, want_h=False)
    assert H2 is None and _rel(E2, E[2:5]) < 1e-15
