"""The multi-rank path on the CPU: two `gloo` ranks (127.0.0.1) shard one shot stream by shot range with
stim_gb300.shard_range, each sampling its share (the oracle stands in for its GPU), and together they
reproduce the single-rank stream exactly; the max-over-ranks timing reduction bench.py uses under torchrun
is checked too."""

import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, text, total, seed, out_dir):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.oracle import OracleCircuit
    from stim_gb300 import shard_range

    first, n = shard_range(total, rank, world)
    d, o, _ = OracleCircuit(text).sample(n, seed, first_shot=first)
    # Variable-size shards: gather padded rows, then the true sizes.
    cap = (total + 127) // 128 * 128
    pad = np.zeros((cap, d.shape[1]), dtype=np.uint8)
    pad[:n] = d
    parts = [torch.zeros((cap, d.shape[1]), dtype=torch.uint8) for _ in range(world)]
    dist.all_gather(parts, torch.from_numpy(pad))
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([n], dtype=torch.int64))
    t = torch.tensor([0.5 * (rank + 1)], dtype=torch.float64)  # this rank's step time
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        got = np.concatenate([p.numpy()[:int(s.item())] for p, s in zip(parts, sizes)])
        np.save(os.path.join(out_dir, "gathered.npy"), got)
        np.save(os.path.join(out_dir, "max_time.npy"), t.numpy())
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("total", [1000, 4096])
def test_two_gloo_ranks_reproduce_the_single_rank_stream(tmp_path, total):
    import torch.multiprocessing as mp

    sys.path.insert(0, ROOT)
    from oracle.oracle import OracleCircuit
    from stim_gb300 import workloads

    text = workloads.code_circuit("surface_code:rotated_memory_z", 3, 3, 0.01)
    seed = 11
    mp.spawn(_worker, args=(2, _free_port(), text, total, seed, str(tmp_path)), nprocs=2, join=True)
    want, _, _ = OracleCircuit(text).sample(total, seed)
    np.testing.assert_array_equal(np.load(tmp_path / "gathered.npy"), want)
    assert float(np.load(tmp_path / "max_time.npy")[0]) == 1.0


def test_shard_range_partitions_whole_blocks():
    from stim_gb300 import shard_range

    for total in [0, 1, 127, 128, 1000, 1 << 20]:
        for world in [1, 2, 3, 8]:
            ranges = [shard_range(total, r, world) for r in range(world)]
            assert sum(n for _, n in ranges) == total
            pos = 0
            for first, n in ranges:
                assert first % 128 == 0 and (n == 0 or first == pos)
                pos = first + n if n else pos
