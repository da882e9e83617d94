"""Replica sharding on the host: the cost partition covers every batched
frame exactly once and balances the estimated cost, and two gloo ranks
(separate processes on CPU) agree on it and reduce timings with max."""
import os
import socket

import pytest

from globalillumination_gb300 import replicas


def test_partition_covers_and_balances():
    costs = [float(c) for c in (9, 7, 6, 5, 5, 4, 3, 3, 2, 1, 1, 1)]
    for world in (1, 2, 3, 4, 8):
        parts = replicas.partition_by_cost(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) <= (4.0 / 3.0) * max(sum(costs) / world, max(costs)) + 1e-9
    assert replicas.partition_by_cost([], 2) == [[], []]
    with pytest.raises(ValueError):
        replicas.partition_by_cost(costs, 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import json

    import torch.distributed as dist

    from globalillumination_gb300 import replicas as rp, scenes

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    frames = scenes.batched_720p(scenes=16, tri_max=50_000)
    costs = [rp.frame_cost(f.triangles, [m.width for m in f.maps], f.camera.width * f.camera.height) for f in frames]
    parts = rp.partition_by_cost(costs, world)
    mine = parts[rank]
    t = rp.max_over_ranks(1.0 + rank, dist)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"parts": parts, "mine": mine, "max_t": t, "n": len(frames)}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_agree(tmp_path):
    import json

    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0 = json.load(open(tmp_path / "rank0.json"))
    r1 = json.load(open(tmp_path / "rank1.json"))
    assert r0["parts"] == r1["parts"]
    assert sorted(r0["mine"] + r1["mine"]) == list(range(r0["n"]))
    assert not set(r0["mine"]) & set(r1["mine"])
    assert r0["max_t"] == r1["max_t"] == 2.0
