"""Sharding host logic over two gloo ranks on the CPU: the reference's
contiguous split, per-shard ray-id offsets that reproduce an unsharded
trace ray by ray (random draws included), and the one all_reduce of
per-field focal moments."""
import os
import socket

import numpy as np
import pytest

import oracle_ref
import shard_worker
from robast_gb300 import configs, shard


@pytest.mark.parametrize("n,world", [(0, 1), (1, 1), (7, 2), (10, 3), (1000, 8), (5, 8)])
def test_shard_range_partitions_in_order(n, world):
    bounds = [shard.shard_range(n, r, world) for r in range(world)]
    assert bounds[0][0] == 0 and bounds[-1][1] == n
    for (a0, a1), (b0, b1) in zip(bounds, bounds[1:]):
        assert a1 == b0 and a0 <= a1
    q = n // world  # the reference's chunk (src/AOpticsManager.cxx:533-541)
    assert all(b1 - b0 == q for b0, b1 in bounds[:-1])


def test_shard_range_rejects_bad_requests():
    for args in ((10, 2, 2), (10, -1, 2), (10, 0, 0), (-1, 0, 1)):
        with pytest.raises(ValueError):
            shard.shard_range(*args)


def test_spot_from_moments():
    rng = np.random.default_rng(0)
    x, y, t = rng.normal(1, 2, 500), rng.normal(-1, 3, 500), rng.uniform(0, 1, 500)
    s = np.array([[500, x.sum(), y.sum(), (x * x).sum(), (y * y).sum(), t.sum()], [0, 0, 0, 0, 0, 0]])
    out = shard.spot_from_moments(s)
    assert out[0, 0] == 500 and np.isclose(out[0, 1], x.mean()) and np.isclose(out[0, 2], y.mean())
    assert np.isclose(out[0, 3], np.sqrt(x.var() + y.var()))
    assert out[1, 0] == 0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_trace_matches_unsharded(tmp_path):
    import torch.multiprocessing as mp

    n, world = 3001, 2
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=shard_worker.run, args=(r, world, port, n, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    parts = [np.load(tmp_path / f"rank{r}.npz") for r in range(world)]

    man, batch = configs.davies_cotton(n_rays=n, n_angles=3)
    n_groups = int(batch["group"].max()) + 1
    st, full = oracle_ref.trace(man, configs.to_array(batch))
    assert st == 0
    status = np.concatenate([p["status"] for p in parts])
    x = np.concatenate([p["x"] for p in parts])
    assert [int(p["first"]) for p in parts] == [shard.shard_range(n, r, world)[0] for r in range(world)]
    # roughness draws are keyed by global ray id: identical fates and points
    np.testing.assert_array_equal(status, full["status"])
    np.testing.assert_array_equal(x, full["x"])
    assert (full["status"] == 3).sum() > n // 4
    want = shard_worker.moments(full["status"], full["x"], full["y"], full["t"], batch["group"], n_groups)
    for p in parts:
        np.testing.assert_allclose(p["total"], want, rtol=1e-12, atol=1e-9)
        assert not np.allclose(p["local"], want)
