"""Rank body of tests/test_shard_gloo.py (a separate module so that spawned
processes can import it).  Each rank traces its shard of a Davies-Cotton
batch (mirror roughness on, so every ray draws random numbers) with the
oracle, sums per-field focal moments over the ranks with one gloo
all_reduce, and writes what it saw to `outdir`."""
import os

import numpy as np


def moments(status, x, y, t, group, n_groups):
    s = np.zeros((n_groups, 6))
    f = status == 3  # RBG_FOCUS
    for g in range(n_groups):
        m = f & (group == g)
        s[g] = (m.sum(), x[m].sum(), y[m].sum(), (x[m] ** 2).sum(), (y[m] ** 2).sum(), t[m].sum())
    return s


def run(rank, world, port, n_rays, outdir):
    import torch
    import torch.distributed as dist

    import oracle_ref
    from robast_gb300 import configs, shard

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        man, batch = configs.davies_cotton(n_rays=n_rays, n_angles=3)
        n_groups = int(batch["group"].max()) + 1
        part, first = shard.shard_batch(batch, rank, world)
        man.ray_id_offset = first
        st, out = oracle_ref.trace(man, configs.to_array(part))
        assert st == 0, st
        local = moments(out["status"], out["x"], out["y"], out["t"], part["group"], n_groups)
        total = shard.allreduce_sum(torch.from_numpy(local.copy())).numpy()
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), first=first, status=out["status"], x=out["x"],
                 y=out["y"], total=total, local=local)
        dist.barrier()
    finally:
        dist.destroy_process_group()
