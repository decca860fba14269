"""Multi-GPU is replicas only: chains are independent (one reference MPI rank
per chain, src/mc_metropolis.cpp:25) and nothing is exchanged on the data path.
The N > 1 host logic of bench.py (rank-distinct chains, max-over-ranks time,
summed end-to-end throughput) runs here as two gloo ranks on the CPU."""
import os
import socket
import sys
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    B = 4
    seeds = bench.chain_seeds(B, rank)
    f = bench.make_chains(B, rank)
    ms, e2e = bench.reduce_replicas(dist, "cpu", 10.0 + rank, 100.0 * (rank + 1))
    np.savez(os.path.join(outdir, f"r{rank}.npz"), seeds=seeds, f=f, ms=ms, e2e=e2e)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_on_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank_main, args=(world, _free_port(), d), nprocs=world, start_method="spawn")
        r = [np.load(os.path.join(d, f"r{k}.npz")) for k in range(world)]
    # each rank holds its own chains: disjoint seeds, different configurations
    assert set(r[0]["seeds"]).isdisjoint(r[1]["seeds"])
    assert list(r[1]["seeds"]) == [s + 4 for s in r[0]["seeds"]]
    assert not np.array_equal(r[0]["f"], r[1]["f"])
    # the job's time is the slowest rank's; end-to-end throughput adds up
    for k in range(world):
        assert float(r[k]["ms"]) == 11.0
        assert float(r[k]["e2e"]) == 300.0


def test_single_replica_matches_the_job():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_replicas(None, "cpu", 5.0, 7.0) == (5.0, 7.0)
    assert bench.chain_seeds(3) == [bench.SEED, bench.SEED + 1, bench.SEED + 2]
