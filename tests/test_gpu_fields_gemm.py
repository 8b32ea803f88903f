"""The far field of many right-hand sides as tensor-core GEMMs (fields_engine
FRICO_FIELDS_GEMM) against the direct multi-column kernels on the same lumped
currents: E within 1e-6 relative (the mixed path's bound on the far field), the
bistatic sigma within 1e-6 of its maximum, column by column; and the choice of
engine by FRICO_FIELDS_AUTO."""
import numpy as np
import pytest

from frico_gb300 import meshes
from frico_gb300.solver import PlaneWave, Simulation

pytestmark = pytest.mark.gpu

GEMM_TOL = 1e-6


def _solved(level, f, ncols, precision):
    m = meshes.icosphere(level)
    sim = Simulation(m, precision=precision)
    sim.compute_matrix(f)
    sim.set_nrhs(ncols)
    th = np.arange(ncols) * np.pi / max(1, ncols - 1)
    for c in range(ncols):
        pw = PlaneWave(float(th[c]), 0.3 * c, 1.0 if c % 2 == 0 else 0.0, 0.0 if c % 2 == 0 else 1.0)
        sim.update_rhs(f, pw, c)
    sim.solve()
    return sim


@pytest.mark.parametrize("level,f,ncols", [(2, 300e6, 5), (3, 450e6, 16)])
def test_fields_gemm_matches_direct(gpu_lib, level, f, ncols):
    sim = _solved(level, f, ncols, "fp64")
    rng = np.random.default_rng(level)
    th = np.arccos(rng.uniform(-1, 1, 777))
    ph = rng.uniform(0, 2 * np.pi, 777)
    pts = meshes.sph2rect(10.0, th, ph)
    sim.set_options(fields_engine=1)
    E_d, _ = sim.eval_fields_multi(pts, want_h=False)
    sig_d = sim.rcs_points_multi(10.0, th, ph)
    sim.set_options(fields_engine=2)
    E_g, _ = sim.eval_fields_multi(pts, want_h=False)
    sig_g = sim.rcs_points_multi(10.0, th, ph)
    for c in range(ncols):
        err = np.linalg.norm(E_g[c] - E_d[c]) / np.linalg.norm(E_d[c])
        assert err < GEMM_TOL, (c, err)
        assert np.abs(sig_g[c] - sig_d[c]).max() < GEMM_TOL * np.abs(sig_d[c]).max(), c


def test_fields_engine_auto_picks_gemm_for_many_columns(gpu_lib):
    """Mixed precision with the default engine evaluates E of many columns as GEMMs
    (results equal the forced GEMM engine's bit for bit) and keeps the direct
    kernels for the FP64 drop-in and whenever H is asked for."""
    sim = _solved(3, 450e6, 8, "mixed")     # 1280 triangles x 16384 points = 2^24.3 pairs
    rng = np.random.default_rng(3)
    pts = meshes.sph2rect(10.0, np.arccos(rng.uniform(-1, 1, 16384)), rng.uniform(0, 2 * np.pi, 16384))
    E_auto, _ = sim.eval_fields_multi(pts, want_h=False)
    sim.set_options(fields_engine=2)
    E_gemm, _ = sim.eval_fields_multi(pts, want_h=False)
    sim.set_options(fields_engine=1)
    E_dir, H_dir = sim.eval_fields_multi(pts, want_h=True)
    assert np.array_equal(E_auto, E_gemm)
    assert not np.array_equal(E_auto, E_dir)
    sim.set_options(fields_engine=0)
    E_h, H_h = sim.eval_fields_multi(pts, want_h=True)
    assert np.array_equal(E_h, E_dir) and np.array_equal(H_h, H_dir)
