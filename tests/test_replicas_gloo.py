"""Multi-GPU form of the path is replicas only (chains are independent, no
exchange): each rank anneals its own seed range and the job's wall time is
the max over ranks.  This runs that bookkeeping as two gloo ranks on the CPU,
with the oracle standing in for each rank's device work."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    import pathlib
    root = pathlib.Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root))
    sys.path.insert(0, str(root / "oracle"))
    import torch
    import oracle as ora
    import rfmf_gb300 as R
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = R.torus(8, 10, signed=True, seed=0)
    setup = bench.chain_setup([g], 4, rank * 4)
    s = setup[0]
    r = ora.anneal(g, s["init"], s["t0s"], s["solver"], [8, 2, 1], [30, 30, 30], nthreads=1)
    elapsed = torch.tensor([float(rank + 1)], dtype=torch.float64)
    dist.all_reduce(elapsed, op=dist.ReduceOp.MAX)
    seeds = torch.tensor(s["seeds"], dtype=torch.int64)
    allseeds = [torch.zeros_like(seeds) for _ in range(world)]
    dist.all_gather(allseeds, seeds)
    q.put((rank, float(elapsed.item()), [int(x) for t in allseeds for x in t],
           [int(x) for x in r["best_vals"]]))
    dist.destroy_process_group()


def test_two_rank_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    # max over ranks, disjoint seed ranges, and rank results independent of the peer
    assert all(o[1] == 2.0 for o in out)
    assert out[0][2] == list(range(8)) and out[1][2] == list(range(8))
    import sys
    import pathlib
    root = pathlib.Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root / "oracle"))
    import oracle as ora
    import rfmf_gb300 as R
    import bench
    g = R.torus(8, 10, signed=True, seed=0)
    s = bench.chain_setup([g], 8, 0)[0]
    alone = ora.anneal(g, s["init"], s["t0s"], s["solver"], [8, 2, 1], [30, 30, 30])
    # rank r's chains use seeds 4r..4r+3 and ladder positions 0..3
    s1 = bench.chain_setup([g], 4, 4)[0]
    r1 = ora.anneal(g, s1["init"], s1["t0s"], s1["solver"], [8, 2, 1], [30, 30, 30])
    assert out[0][3] == [int(x) for x in alone["best_vals"][:4]]
    assert out[1][3] == [int(x) for x in r1["best_vals"]]
