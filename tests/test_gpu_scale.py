"""Parity at the benchmark configurations' own scale, against the reference's
own kernel run live on the same GPU (oracle/_ref/anneal_kernels.cubin, built
from its sources; launched as the reference's host code launches it, one
graph per launch).  Every chain is compared: end spins, best spins, final and
best cut values, all identical (integer work, zero tolerance).

* the mid-size configuration: 50x60 torus (+-1) and Erdos-Renyi n = 2000 mean
  degree 19 (+-1), 1024 chains each (raw seeds 0..1023, t0 ladder
  35..400 round-robin), the default phases 128..1 at 1000 sweeps each, run as
  the bench runs it: both graphs in ONE batch;
* the large sparse configuration: 100x200 torus (+-1), random tree
  n = 10000 (+1), Erdos-Renyi n = 5000 mean degree 5 (+-1), 256 chains each,
  1000 sweeps per phase, one batch (the torus's CSR is walked in HBM);
* a batched-configuration mix in one batch whose graphs fall into every
  launch class the planner has: 16-bit and 32-bit shared-memory CSRs, HBM
  walks, int8 and int32 gains, the int64 score path, one and several warps
  per chain.

The comparison cases mirror the reference's chain-isolation test
(tests/test_chain_isolation.sh:66-90,109-132): a chain's output inside a
large launch equals the reference's output for that chain."""
import numpy as np
import pytest

from conftest import chains_for

pytestmark = pytest.mark.gpu

LADDER = [35.0, 50.0, 70.0, 100.0, 140.0, 200.0, 280.0, 400.0]
PHASES = [128, 64, 32, 16, 8, 4, 2, 1]


def _weighted(rfmf, n, avg_degree, wmax, seed, name):
    rng = np.random.default_rng(seed)
    m = int(n * avg_degree / 2)
    u = rng.integers(0, n, m)
    v = rng.integers(0, n, m)
    keep = u != v
    w = rng.integers(1, wmax + 1, int(keep.sum())) * rng.choice([-1, 1], int(keep.sum()))
    return rfmf.csr_from_edges(u[keep], v[keep], w, name=name)


def _batch_vs_reference(rfmf, ctx, refgpu, specs, phases, iters):
    """specs: list of (graph, seeds, t0s).  Runs every chain in one batch and
    each graph's chains through the reference kernel; returns the batch's
    plan after checking every chain."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    dgs, gl, ini, sol, t0 = [], [], [], [], []
    setups = []
    for g, seeds, t0s in specs:
        init, solver = chains_for(g, seeds)
        setups.append((g, init, solver, t0s))
        dg = rfmf.DeviceGraph(ctx, g)
        dgs.append(dg)
        gl += [dg] * len(seeds)
        ini += list(init)
        sol += solver
        t0 += list(t0s)
    b = rfmf.Batch(ctx, gl, t0, sol, ini, phases, iters)
    b.run(sum(iters))
    info = b.info()
    out = b.read()
    b.close()
    c0 = 0
    for g, init, solver, t0s in setups:
        C = init.shape[0]
        ref = refgpu.run(g, init, t0s, solver, phases, iters, sms)
        sl = slice(c0, c0 + C)
        assert np.array_equal(np.stack(out["end_spins"][sl]), ref["end_spins"]), g.name
        assert np.array_equal(np.stack(out["best_spins"][sl]), ref["best_spins"]), g.name
        assert np.array_equal(out["cur_vals"][sl], ref["cur_vals"]), g.name
        assert np.array_equal(out["best_vals"][sl], ref["best_vals"]), g.name
        c0 += C
    for dg in dgs:
        dg.close()
    return info


def test_mid_size_configuration_1024_chains(rfmf, ctx, refgpu):
    seeds = list(range(1024))
    t0s = [LADDER[i % 8] for i in range(1024)]
    specs = [(rfmf.torus(50, 60, signed=True, seed=0, name="torus50x60"), seeds, t0s),
             (rfmf.erdos_renyi_degree(2000, 19, signed=True, seed=0, name="er2000_d19"), seeds, t0s)]
    _batch_vs_reference(rfmf, ctx, refgpu, specs, PHASES, [1000] * 8)


def test_large_sparse_configuration_256_chains(rfmf, ctx, refgpu):
    seeds = list(range(256))
    t0s = [LADDER[i % 8] for i in range(256)]
    specs = [(rfmf.torus(100, 200, signed=True, seed=0, name="torus100x200"), seeds, t0s),
             (rfmf.random_tree(10000, seed=0, name="tree10000"), seeds, t0s),
             (rfmf.erdos_renyi_sparse(5000, 5, signed=True, seed=0, name="er5000_d5"), seeds, t0s)]
    info = _batch_vs_reference(rfmf, ctx, refgpu, specs, PHASES, [1000] * 8)
    assert info["launch_classes"] >= 2


def test_every_launch_class_in_one_batch(rfmf, ctx, refgpu):
    C = 64
    seeds = list(range(7000, 7000 + C))
    ladder = [LADDER[i % 8] for i in range(C)]
    specs = [
        (rfmf.erdos_renyi_degree(1200, 8, signed=True, seed=1, name="er1200_d8"), seeds, ladder),
        (rfmf.torus(40, 50, seed=2, name="torus40x50_p1"), seeds, ladder),
        (rfmf.planar_like(3000, 11.7, signed=True, seed=3, name="planar3000"), seeds, ladder),
        # |w| <= 30 on mean degree 12: B > 127, int32 gains, 32-bit entries
        (_weighted(rfmf, 900, 12, 30, seed=4, name="er900_w30"), seeds,
         [20.0 * t for t in ladder]),
        # 100x200 torus: its CSR does not fit beside the chains, HBM walks
        (rfmf.torus(100, 200, signed=True, seed=5, name="torus100x200"), seeds, ladder),
        # n = 20000 sparse +1 graph: HBM walks
        (rfmf.erdos_renyi_sparse(20000, 5, seed=6, name="er20000_d5"), seeds, ladder),
        # t0 = 0.05 on half its chains: the compact int32 key would overflow,
        # so this graph's chains take the int64 score path
        (rfmf.erdos_renyi(600, 0.03, signed=True, seed=7, name="er600_int64"), seeds,
         [0.05 if i % 2 else 35.0 for i in range(C)]),
    ]
    info = _batch_vs_reference(rfmf, ctx, refgpu, specs, PHASES, [250] * 8)
    assert info["launch_classes"] >= 4, info
