"""Function-batch sharding on two CPU ranks (gloo, world_size 2): each rank transforms its
own block of functions with the oracle, rank 0 gathers them, and the result equals the
single-process computation; the max-over-ranks reduction of step times (the bench's
multi-GPU timing rule) returns the slower rank's time."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT, so3_coeffs

L = 3
NFN = 5


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_path):
    import sys

    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    from fftso3_gb300 import shard
    from oracle import oracle as O

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert shard.rank_world() == (rank, world)
        block = shard.partition(NFN, world, rank)
        local = np.stack([O.so3_forward_complex(L, O.so3_inverse_complex_grid(L, so3_coeffs(L, seed=2200 + i)))
                          for i in block]) if len(block) else np.zeros((0, 0), complex)
        full = shard.gather_to_rank0(local, NFN)
        tmax = shard.max_over_ranks(10.0 + rank)
        if rank == 0:
            np.save(out_path, full)
            with open(out_path + ".t", "w") as f:
                f.write(str(tmax))
    finally:
        dist.destroy_process_group()


def test_partition_covers_the_batch():
    from fftso3_gb300 import shard
    for n in (0, 1, 5, 17):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in shard.partition(n, world, r)]
            assert got == list(range(n))
            sizes = [len(shard.partition(n, world, r)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.partition(3, 2, 2)


def test_two_rank_gloo_shard(tmp_path, oracle):
    import torch.multiprocessing as mp

    out = str(tmp_path / "full.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    full = np.load(out)
    ref = np.stack([oracle.so3_forward_complex(L, oracle.so3_inverse_complex_grid(L, so3_coeffs(L, seed=2200 + i)))
                    for i in range(NFN)])
    # the oracle merges its OpenMP partial sums in thread order, so equal to rounding only
    assert full.shape == ref.shape and np.allclose(full, ref, rtol=1e-13, atol=1e-15)
    assert float(open(out + ".t").read()) == 11.0
