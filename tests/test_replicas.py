"""Runs over several GPUs: the member partition and the timing reduction, on two
gloo ranks on the CPU (the data path has no collective; these are the only
multi-rank pieces)."""

import os
import socket

import numpy as np
import pytest

from hypar_gb300 import replicas as R


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_members_partitions_and_balances():
    from hypar_gb300 import cases as C

    sizes = C.ensemble_sizes(64, 20261203)
    cells = [n * n for n in sizes]
    for ws in (1, 2, 3, 4, 8):
        parts = R.shard_members(cells, ws)
        assert len(parts) == ws
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(cells)))  # every member exactly once
        loads = [sum(cells[k] for k in p) for p in parts]
        # LPT bound: no rank above the mean by more than the largest member
        assert max(loads) - sum(loads) / ws <= max(cells)
        assert R.shard_members(cells, ws) == parts  # deterministic
    assert R.shard_members([5, 5, 5], 1) == [[0, 1, 2]]
    assert R.shard_members([1, 9], 3) == [[1], [0], []]
    with pytest.raises(ValueError):
        R.shard_members([1], 0)
    with pytest.raises(ValueError):
        R.aggregate_rate(1.0, 1, 0.0)
    assert R.aggregate_rate(10.0, 4, 2.0) == 20.0


def _rank_main(rank, ws, port, out_dir):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    from hypar_gb300 import cases as C

    sizes = C.ensemble_sizes(16, 7)
    parts = R.shard_members([n * n for n in sizes], ws)
    mine = parts[rank]
    # a rank's "timed interval" grows with its share, as a slowest-rank proxy
    t_mine = 1e-3 * sum(sizes[k] ** 2 for k in mine) / 1e5 + rank * 1e-6
    t_max = R.max_over_ranks(t_mine, dist)
    dist.barrier()
    np.save(os.path.join(out_dir, f"rank{rank}.npy"),
            np.array([t_mine, t_max] + [float(k) for k in mine], dtype=np.float64))
    dist.destroy_process_group()


def test_two_gloo_ranks_partition_and_max(tmp_path):
    import torch.multiprocessing as mp

    ws = 2
    mp.spawn(_rank_main, args=(ws, _free_port(), str(tmp_path)), nprocs=ws, join=True)
    rows = [np.load(tmp_path / f"rank{r}.npy") for r in range(ws)]
    t = [r[0] for r in rows]
    assert all(r[1] == max(t) for r in rows)  # every rank sees the slowest rank's time
    got = sorted(int(k) for r in rows for k in r[2:])
    assert got == list(range(16))  # the ranks' shares cover the ensemble exactly once
