"""Batched frequency sweep (frico_gpu_sweep) against single-frequency calls and
the oracle, on the bowtie of the sweep workload (N ~ 500, feed + 3 plane waves)."""
import numpy as np
import pytest

from frico_gb300 import meshes
from frico_gb300._abi import FricoError
from frico_gb300.solver import DeltaGap, PlaneWave, Simulation

DEG = np.pi / 180
PLANE_WAVES = (PlaneWave(0.0, 0.0, 1.0, 0.0), PlaneWave(45 * DEG, 0.0, 1.0, 0.0), PlaneWave(90 * DEG, 90 * DEG, 0.0, 1.0))
FEED = DeltaGap((meshes.FEED_TAG,), 1.0)


@pytest.fixture(scope="module")
def bowtie500():
    return meshes.bowtie_preset(500)


def _points(n=6):
    th = np.linspace(10, 170, n) * DEG
    return meshes.sph2rect(10.0, th, 0.3 + 0 * th)


def _single(sim, f, pts):
    """The sweep's per-frequency pipeline through the single-frequency calls."""
    sim.compute_matrix(f)
    sim.set_nrhs(4)
    sim.update_rhs(f, FEED, 0)
    for c, pw in enumerate(PLANE_WAVES):
        sim.update_rhs(f, pw, c + 1)
    I = sim.solve()
    pv = sim.port_values(FEED)
    E = np.stack([sim.eval_fields(pts, col=c)[0] for c in range(4)])
    return I.T.copy(), pv, E


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sweep_equals_single_frequency_calls(gpu_lib, bowtie500, precision):
    freqs = meshes.sweep_frequencies(200e6, 800e6, 5)
    pts = _points()
    sim = Simulation(bowtie500, precision=precision)
    out = sim.sweep(freqs, FEED, PLANE_WAVES, pts, lanes=3, currents=True)
    rep = out["report"]
    assert rep["nrhs"] == 4 and rep["lanes"] == 3 and rep["not_converged"] == 0
    ref = Simulation(bowtie500, precision=precision)
    for i, f in enumerate(freqs):
        I, pv, E = _single(ref, f, pts)
        np.testing.assert_array_equal(out["I"][i], I)
        # the sweep evaluates all columns in one multi-column field pass (FP64); the
        # single-column calls of the mixed path sum in double-float (2^-47 per operation)
        assert np.abs(out["E"][i] - E).max() <= 1e-11 * np.abs(E).max()
        assert out["port"][i]["impedance"] == pv["impedance"]


@pytest.mark.gpu
def test_sweep_fp64_matches_oracle(gpu_lib, bowtie500):
    from oracle import Oracle
    o = Oracle(bowtie500)
    freqs = np.array([350e6, 610e6])
    sim = Simulation(bowtie500, precision="fp64")
    out = sim.sweep(freqs, FEED, PLANE_WAVES[:1], currents=True)
    for i, f in enumerate(freqs):
        Z = o.compute_matrix(f)
        V = np.stack([o.rhs_delta_gap(f, [meshes.FEED_TAG]), o.rhs_plane_wave(f, 0.0, 0.0, 1.0, 0.0)], axis=1)
        Ir = o.solve(Z, V)
        err = np.linalg.norm(out["I"][i].T - Ir) / np.linalg.norm(Ir)
        assert err < 1e-9
        pr = o.port_values(Ir[:, 0], o.rwg(), [meshes.FEED_TAG])
        assert abs(out["port"][i]["impedance"] - pr["impedance"]) / abs(pr["impedance"]) < 1e-9


@pytest.mark.gpu
def test_sweep_autotuned_lanes_give_the_same_results(gpu_lib, bowtie500):
    freqs = meshes.sweep_frequencies(200e6, 800e6, 160)
    sim = Simulation(bowtie500, precision="mixed")
    tuned = sim.sweep(freqs, FEED, PLANE_WAVES)
    assert tuned["report"]["autotuned"] == 1 and tuned["report"]["lanes"] >= 1
    one = sim.sweep(freqs, FEED, PLANE_WAVES, lanes=1)
    assert one["report"]["autotuned"] == 0
    assert [p["impedance"] for p in tuned["port"]] == [p["impedance"] for p in one["port"]]


@pytest.mark.gpu
def test_sweep_argument_errors(gpu_lib, bowtie500):
    sim = Simulation(bowtie500)
    with pytest.raises(FricoError) as e:
        sim.sweep([300e6])                     # no right-hand side
    assert e.value.code == -1
    with pytest.raises(FricoError) as e:
        sim.sweep([300e6, -1.0], FEED)          # bad frequency
    assert e.value.code == -1
