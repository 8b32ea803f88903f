"""frico_gpu_eval_fields_noalloc (device buffers, fixed scratch) against
frico_gpu_eval_fields on the same lumped currents.

Collected last on purpose: it must hold after every other GPU test has run in
the same process (the scratch array is shared by all contexts on a device).
"""
import ctypes as C

import numpy as np
import pytest

from frico_gb300 import meshes
from frico_gb300.solver import PlaneWave, Simulation

MAX_POINTS = (1 << 18) // 6   # fixed 4 MiB scratch of complex128 partial sums, 6 per point and chunk


def _points(npts: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((npts, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.ascontiguousarray(d * rng.uniform(2.0, 20.0, (npts, 1)))


def _solved_sphere():
    m = meshes.icosphere(3)
    f = 450e6
    sim = Simulation(m, precision="mixed")
    sim.compute_matrix(f)
    sim.set_nrhs(1)
    sim.update_rhs(f, PlaneWave(0.0, 0.0, 1.0, 0.0))
    sim.solve()
    sim.lump_currents(0)
    return sim


def _noalloc(sim, P_dev, E_dev, H_dev, npts):
    return sim.lib.frico_gpu_eval_fields_noalloc(sim.ctx, 0, npts, C.c_void_p(P_dev), C.c_void_p(E_dev),
                                                 C.c_void_p(H_dev))


@pytest.mark.gpu
@pytest.mark.parametrize("npts", [362, 8000, MAX_POINTS])
def test_noalloc_matches_eval_fields_twice(gpu_lib, npts):
    import torch
    sim = _solved_sphere()
    pts = _points(npts, 7 + npts)
    E_ref, H_ref = sim.eval_fields(pts)
    P_dev = torch.from_numpy(pts).to("cuda:0")
    E_dev = torch.empty((npts, 3, 2), dtype=torch.float64, device="cuda:0")
    H_dev = torch.empty((npts, 3, 2), dtype=torch.float64, device="cuda:0")
    for _ in range(2):   # two calls in a row through the same scratch
        E_dev.fill_(float("nan"))
        H_dev.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = _noalloc(sim, P_dev.data_ptr(), E_dev.data_ptr(), H_dev.data_ptr(), npts)
        assert rc == 0, sim.lib.frico_gpu_last_error(sim.ctx).decode()
        torch.cuda.synchronize()
        E = E_dev.cpu().numpy().view(np.complex128)[..., 0]
        H = H_dev.cpu().numpy().view(np.complex128)[..., 0]
        assert np.isfinite(E).all() and np.isfinite(H).all()
        assert np.abs(E - E_ref).max() <= 1e-12 * np.abs(E_ref).max()
        assert np.abs(H - H_ref).max() <= 1e-12 * np.abs(H_ref).max()


@pytest.mark.gpu
def test_noalloc_rejects_before_launch(gpu_lib):
    import torch
    sim = _solved_sphere()
    npts = MAX_POINTS + 1
    P_dev = torch.zeros((npts, 3), dtype=torch.float64, device="cuda:0")
    E_dev = torch.empty((npts, 3, 2), dtype=torch.float64, device="cuda:0")
    # over the scratch limit
    assert _noalloc(sim, P_dev.data_ptr(), E_dev.data_ptr(), 0, npts) == -1
    assert b"scratch" in sim.lib.frico_gpu_last_error(sim.ctx)
    # host pointers are refused
    host = np.zeros((16, 3))
    assert _noalloc(sim, host.ctypes.data, E_dev.data_ptr(), 0, 16) == -1
    assert b"device" in sim.lib.frico_gpu_last_error(sim.ctx)
    # misaligned views (one double past an aligned buffer) are refused before any launch
    assert _noalloc(sim, P_dev.data_ptr(), E_dev.data_ptr() + 8, 0, 16) == -1
    assert b"aligned" in sim.lib.frico_gpu_last_error(sim.ctx)
    assert _noalloc(sim, P_dev.data_ptr() + 4, E_dev.data_ptr(), 0, 16) == -1
    assert b"aligned" in sim.lib.frico_gpu_last_error(sim.ctx)
    # currents of the column not lumped: a fresh solve clears the lumped column
    sim.solve()
    assert _noalloc(sim, P_dev.data_ptr(), E_dev.data_ptr(), 0, 16) == -6
    torch.cuda.synchronize()
