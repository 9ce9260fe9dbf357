"""Multi-GPU is replicas only: every operation of the path is independent per ciphertext and keys
are read-only, so N ranks run N independent copies of the workload with no data-path collective;
the only cross-rank steps are the barrier around the timed region and the max-over-ranks time.
This covers that host logic with two gloo ranks on the CPU, each running a small oracle key
switch as its replica."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from oracle import oracle as O
        # a replica: the same seeded key switch on every rank (independent work, same inputs)
        mods = O.create_coeff_modulus(4096, [60, 40, 40, 60])
        oc = O.Context(12, mods, 3, 1)
        rng = np.random.default_rng(5)
        ct = O.random_residues(rng, mods[:3], 4096, 2)
        c2 = O.random_residues(rng, mods[:3], 4096, 1)[0]
        key = O.random_residues(rng, mods, 4096, 2 * 3).reshape(3, 2, 4, 4096)
        res = oc.keyswitch(3, ct, c2, key)
        digest = int(np.bitwise_xor.reduce(res.ravel()))
        dist.barrier()
        t = 0.5 + rank  # this rank's timed region (s)
        tmax = bench.max_over_ranks(t, world, "cpu")
        value = bench.replica_throughput(10, world, tmax)
        gathered = [None] * world
        dist.all_gather_object(gathered, digest)
        out[rank] = (tmax, value, len(set(gathered)))
    finally:
        dist.destroy_process_group()


def test_replicas_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(world):
        tmax, value, distinct = out[r]
        assert tmax == pytest.approx(1.5)          # the slowest rank's time
        assert value == pytest.approx(10 * 2 / 1.5)  # all ranks' operations over that time
        assert distinct == 1                        # replicas computed the same words
