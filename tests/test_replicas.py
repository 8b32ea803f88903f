"""Multi-replica layout (one process per GPU, no data-path collective), tested
on the host with gloo ranks: frequency sharding, the barrier / max-of-times
bookkeeping and the in-order gather of per-frequency results."""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from frico_gb300.replicas import ReplicaGroup, shard, shard_bounds  # noqa: E402


@pytest.mark.parametrize("n,world", [(0, 1), (1, 2), (7, 2), (256, 8), (10, 3), (3, 4)])
def test_shard_bounds_partition(n, world):
    blocks = [shard_bounds(n, r, world) for r in range(world)]
    assert blocks[0][0] == 0 and blocks[-1][1] == n
    for (lo, hi), (lo2, _) in zip(blocks, blocks[1:]):
        assert hi == lo2
    sizes = [hi - lo for lo, hi in blocks]
    assert max(sizes) - min(sizes) <= 1
    assert [x for r in range(world) for x in shard(list(range(n)), r, world)] == list(range(n))


def test_shard_bounds_rejects_bad_rank():
    with pytest.raises(ValueError):
        shard_bounds(4, 2, 2)
    with pytest.raises(ValueError):
        shard_bounds(4, 0, 0)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _impedance_sweep(freqs):
    """Per-frequency input impedance of the strip dipole, computed by the
    oracle (CPU restatement of FRICO's antenna path)."""
    sys.path.insert(0, str(ROOT))
    from frico_gb300 import meshes
    from oracle import Oracle
    m = meshes.strip_dipole()
    o = Oracle(m)
    out = []
    for f in freqs:
        Z = o.compute_matrix(f)
        V = o.rhs_delta_gap(f, [meshes.FEED_TAG])
        I = o.solve(Z, V)
        pv = o.port_values(I, o.rwg(), [meshes.FEED_TAG])
        out.append([pv["impedance"], pv["current"]])
    return np.array(out, dtype=np.complex128).reshape(len(freqs), 2)


def _rank_main(rank, world, port, freqs, outdir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    g = ReplicaGroup(world, rank, backend="gloo")
    try:
        mine = shard(freqs, rank, world)
        g.barrier()
        rows = _impedance_sweep(mine)
        t = g.max(float(rank + 1))          # max over ranks
        total = g.sum(float(len(mine)))     # units processed by all ranks
        full = g.gather_rows(rows, len(freqs))
        g.barrier()
        np.savez(Path(outdir) / f"rank{rank}.npz", full=full, tmax=t, total=total)
    finally:
        g.close()


def test_two_rank_frequency_sweep_gloo(tmp_path):
    freqs = list(np.linspace(250e6, 350e6, 5))
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, freqs, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
        assert p.exitcode == 0
    serial = _impedance_sweep(freqs)
    for r in range(2):
        d = np.load(tmp_path / f"rank{r}.npz")
        assert float(d["tmax"]) == 2.0
        assert float(d["total"]) == len(freqs)
        np.testing.assert_array_equal(d["full"], serial)   # bit-identical: same code, same order


def test_single_replica_is_a_no_op():
    g = ReplicaGroup(1, 0)
    rows = np.arange(6, dtype=np.complex128).reshape(3, 2)
    assert g.max(3.5) == 3.5 and g.sum(2.0) == 2.0
    assert g.gather_rows(rows, 3) is not None and np.array_equal(g.gather_rows(rows, 3), rows)
    g.barrier()
    g.close()
