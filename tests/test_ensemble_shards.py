"""Sharding ensemble members over ranks (no GPU): the member split and the
host-side gather of per-member rows over a world-size-2 gloo process group."""
import os
import socket

import pytest

from palinstrophy_gb300.ensemble_shards import gather_rows, member_range, shard_members


@pytest.mark.parametrize("n,world", [(0, 1), (1, 2), (5, 2), (96, 2), (96, 3), (96, 8), (7, 8), (100, 7)])
def test_member_range_partitions(n, world):
    seen = []
    sizes = []
    for r in range(world):
        lo, hi = member_range(n, r, world)
        assert 0 <= lo <= hi <= n
        seen.extend(range(lo, hi))
        sizes.append(hi - lo)
    assert seen == list(range(n))  # contiguous, disjoint, in rank order
    assert max(sizes) - min(sizes) <= 1


def test_member_range_rejects_bad_rank():
    with pytest.raises(ValueError):
        member_range(4, 2, 2)
    with pytest.raises(ValueError):
        member_range(4, 0, 0)


def test_shard_members_slices():
    members = list(range(10, 20))
    assert shard_members(members, 0, 3) + shard_members(members, 1, 3) + shard_members(members, 2, 3) == members


def test_gather_without_process_group_is_identity():
    assert gather_rows([{"member": 3}]) == [{"member": 3}]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, n, out_path):
    import json
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, hi = member_range(n, rank, world)
        rows = [{"member": m, "rank": rank, "value": m * m} for m in range(lo, hi)]
        got = gather_rows(rows)
        if rank == 0:
            with open(out_path, "w") as f:
                json.dump(got, f)
        else:
            assert got is None
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_gather_rows_two_ranks_gloo(tmp_path):
    import json
    import torch.multiprocessing as mp
    world, n = 2, 7
    out = str(tmp_path / "rows.json")
    mp.spawn(_worker, args=(world, _free_port(), n, out), nprocs=world, join=True)
    with open(out) as f:
        rows = json.load(f)
    assert [r["member"] for r in rows] == list(range(n))
    assert [r["rank"] for r in rows] == [0, 0, 0, 0, 1, 1, 1]
    assert all(r["value"] == r["member"] ** 2 for r in rows)
