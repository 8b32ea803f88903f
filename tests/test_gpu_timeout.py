"""A device-side wait that runs out returns FRICO_GPU_ETIMEOUT and leaves the
context usable.

The wait is made to run out by a limit far below any real dependency time
(`wait_limit_cycles` = 200 SM cycles): the chained triangular solves of the
refinement wait that long for the block solved before them, give up, record
the timeout in the device status word and return. Nothing faults or hangs:
every wait checks its own clock and the shared status word.
"""
import numpy as np
import pytest

from frico_gb300 import _abi, meshes
from frico_gb300._abi import FricoError
from frico_gb300.solver import PlaneWave, Simulation

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_short_wait_limit_times_out_then_context_solves(gpu_lib, precision):
    m = meshes.icosphere(3)
    f = 450e6
    pw = PlaneWave(0.0, 0.0, 1.0, 0.0)
    ref = Simulation(m, precision=precision)
    ref.compute_matrix(f)
    ref.update_rhs(f, pw)
    I_ref = ref.solve()

    sim = Simulation(m, precision=precision, wait_limit_cycles=200)
    sim.compute_matrix(f)
    sim.update_rhs(f, pw)
    with pytest.raises(FricoError) as ei:
        sim.solve()
    assert ei.value.code == _abi.ETIMEOUT, str(ei.value)
    assert "timed out" in str(ei.value)
    # the default limit again: the same context solves correctly. A timeout in the chained
    # solves keeps the factors; one in the pivoted panel's grid barrier stops a factorisation
    # that works in place, after which a solve without a new fill is refused as out of order
    sim.set_options(wait_limit_cycles=0)
    try:
        I = sim.solve()
    except FricoError as e:
        assert e.code == _abi.ESTATE, str(e)
        sim.compute_matrix(f)
        I = sim.solve()
    assert np.linalg.norm(I - I_ref) <= 1e-12 * np.linalg.norm(I_ref)
