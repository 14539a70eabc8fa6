"""The multi-GPU path is replicas: contiguous slices of the global batch per rank, outcomes gathered
on the host, the step time is the maximum over ranks.  Two gloo ranks on the CPU (no GPU needed)
check the slicing, the gather and the max; each rank checks its slice with the oracle as a stand-in
for the device call."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import pyoracle
    from plainmp_gb300 import replicas
    from plainmp_gb300 import workloads as W

    n = 1001
    a, b = replicas.shard(n, rank, world)
    Q = W.chain7_configs(n, seed=5)[a:b]
    _, oc, _ = pyoracle.make_constraint(W.chain7_robot(), W.chain7_scene())
    ok = oc.is_valid(Q)
    allok = replicas.gather_outcomes(ok, dist)
    t = replicas.max_over_ranks(10.0 + rank, dist)
    np.save(os.path.join(out_dir, f"r{rank}.npy"), np.concatenate([[a, b, t], allok.astype(np.float64)]))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_covers_the_batch():
    from plainmp_gb300.replicas import shard

    for n in (0, 1, 7, 1001):
        for world in (1, 2, 3, 8):
            parts = [shard(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(10, 2, 2)


def test_two_gloo_ranks(tmp_path, oracle):
    import torch.multiprocessing as mp

    from plainmp_gb300 import workloads as W

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn", join=True)
    _, oc, _ = oracle.make_constraint(W.chain7_robot(), W.chain7_scene())
    ref = oc.is_valid(W.chain7_configs(1001, seed=5))
    spans = []
    for r in range(world):
        v = np.load(tmp_path / f"r{r}.npy")
        spans.append((int(v[0]), int(v[1])))
        assert v[2] == 11.0  # max over ranks of 10 + rank
        assert np.array_equal(v[3:].astype(np.uint8), ref)  # every rank holds the gathered outcomes
    assert spans == [(0, 501), (501, 1001)]
