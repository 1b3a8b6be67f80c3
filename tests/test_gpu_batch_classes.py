"""Batches whose graphs fall into several launch classes (gain width, CSR
format, warps per chain, score path): each class runs as its own
persistent launch on its own stream, and every chain must still equal a
standalone anneal of its graph bit for bit -- also when the windows are
replayed from a captured CUDA graph."""
import numpy as np
import pytest

from conftest import chains_for

pytestmark = pytest.mark.gpu


def _graphs(rfmf):
    heavy = rfmf.erdos_renyi(260, 0.05, signed=True, seed=6)
    heavy.weight = heavy.weight * 9          # B > 127: int32 gains
    return [
        rfmf.erdos_renyi(300, 0.04, signed=True, seed=1),     # small, unit16
        rfmf.torus(60, 150, signed=True, seed=2),             # n = 9000: W = 2
        rfmf.planar_like(1500, seed=3),                       # +1 weights
        heavy,
    ]


def _run(rfmf, ctx, graphs, t0_of, phases, iters, use_graph):
    dgs = [rfmf.DeviceGraph(ctx, g) for g in graphs]
    per = []
    gl, ini, sol, t0 = [], [], [], []
    for k, g in enumerate(graphs):
        seeds = list(range(1000 * k, 1000 * k + 12))
        init, solver = chains_for(g, seeds)
        ts = [t0_of(k, i) for i in range(12)]
        per.append((init, solver, ts))
        gl += [dgs[k]] * 12
        ini += list(init)
        sol += solver
        t0 += ts
    b = rfmf.Batch(ctx, gl, t0, sol, ini, phases, iters)
    info = b.info()
    total = sum(i for p, i in zip(phases, iters) if p)
    if use_graph:
        b.run_graph(total // 4, launches=2, replays=2)
    else:
        b.run(total // 3)
        b.run(total)
    r = b.read()
    b.close()
    return dgs, per, info, r


@pytest.mark.parametrize("use_graph", [False, True])
def test_multi_class_batch_matches_standalone(rfmf, ctx, use_graph):
    graphs = _graphs(rfmf)
    phases, iters = [64, 8, 1], [200, 200, 200]
    # graph 0 chains 0-3 at a tiny t0 force the int64 score path for graph 0
    t0_of = lambda k, i: 0.004 if (k == 0 and i < 4) else 50.0 + 10 * i
    dgs, per, info, r = _run(rfmf, ctx, graphs, t0_of, phases, iters, use_graph)
    assert info["launch_classes"] >= 3, info
    for k, g in enumerate(graphs):
        init, solver, ts = per[k]
        ref = rfmf.anneal_gpu(ctx, dgs[k], g.max_weighted_degree(), init, ts, phases, iters, solver)
        sl = slice(12 * k, 12 * k + 12)
        assert np.array_equal(np.stack(r["best_spins"][sl]), ref.best_spins), k
        assert np.array_equal(np.stack(r["end_spins"][sl]), ref.end_spins), k
        assert np.array_equal(r["best_vals"][sl], ref.best_vals), k
        assert np.array_equal(r["cur_vals"][sl], ref.final_vals), k


def test_auto_warps_follow_chain_count(rfmf, ctx):
    """Few chains per SM get wider warp groups; enough chains to fill the SMs
    run one warp each.  Results do not depend on the width (covered by the
    schedule-invariance knobs); this checks the plan."""
    g = rfmf.erdos_renyi(800, 0.06, seed=0)
    dg = rfmf.DeviceGraph(ctx, g)
    sms = ctx.info()["sm_count"]
    widths = {}
    for C in (32, 8 * sms):
        init, solver = chains_for(g, list(range(C)))
        b = rfmf.Batch(ctx, [dg] * C, [70.0] * C, solver, list(init), [8, 1], [4, 4])
        widths[C] = b.info()["threads_per_chain"]
        b.close()
    assert widths[32] > 32, widths
    assert widths[8 * sms] == 32, widths


def test_widening_when_shared_memory_limits_residency(rfmf, ctx):
    """16 chains per SM of ER n = 5000 (mean degree 5): with one warp each
    only ~12 fit an SM's shared memory beside the graph, so the planner gives
    each chain two warps (16 warps resident); the same graph with 8 chains
    per SM keeps them all resident at one warp each."""
    g = rfmf.erdos_renyi_sparse(5000, 5, signed=True, seed=0)
    dg = rfmf.DeviceGraph(ctx, g)
    sms = ctx.info()["sm_count"]
    widths = {}
    for C in (8 * sms, 16 * sms):
        init, solver = chains_for(g, list(range(C)))
        b = rfmf.Batch(ctx, [dg] * C, [70.0] * C, solver, list(init), [8, 1], [4, 4])
        widths[C] = b.info()["threads_per_chain"]
        b.close()
    assert widths[16 * sms] == 64, widths
    assert widths[8 * sms] == 32, widths


def test_items_resized_per_phase_keep_results(rfmf, ctx, oracle):
    """Two graphs in one class whose relative cost flips between phases (a
    dense ER graph costs more per sweep at P = 128, the larger torus at
    P = 1): windows that cross phase boundaries are cut there and each piece
    runs with items sized from costs learned at its own P (synchronised
    windows of 300 sweeps, so costs are learned between them).  Every chain
    still equals the oracle."""
    graphs = [rfmf.torus(30, 30, signed=True, seed=4), rfmf.erdos_renyi(600, 0.05, signed=True, seed=5)]
    phases, iters = [128, 16, 1], [400, 400, 400]
    dgs = [rfmf.DeviceGraph(ctx, g) for g in graphs]
    gl, ini, sol, t0, per = [], [], [], [], []
    for k, g in enumerate(graphs):
        init, solver = chains_for(g, list(range(500 * k, 500 * k + 96)))
        ts = [35.0 + 15 * (i % 8) for i in range(96)]
        per.append((init, solver, ts))
        gl += [dgs[k]] * 96
        ini += list(init)
        sol += solver
        t0 += ts
    b = rfmf.Batch(ctx, gl, t0, sol, ini, phases, iters)
    assert b.info()["launch_classes"] == 1
    for _ in range(4):
        b.run_timed(300)
    info = b.info()
    r = b.read()
    b.close()
    assert info["balanced"] == 1, info
    # windows [0,300) [300,600) [600,900) [900,1200) over phases ending at
    # 400, 800, 1200: cut into 1 + 2 + 2 + 1 launches of the one class
    assert info["launches"] == 6, info
    for k, g in enumerate(graphs):
        init, solver, ts = per[k]
        ref = oracle.anneal(g, init, ts, solver, phases, iters)
        sl = slice(96 * k, 96 * k + 96)
        assert np.array_equal(np.stack(r["end_spins"][sl]), ref["end_spins"]), k
        assert np.array_equal(np.stack(r["best_spins"][sl]), ref["best_spins"]), k
        assert np.array_equal(r["cur_vals"][sl], ref["cur_vals"]), k
        assert np.array_equal(r["best_vals"][sl], ref["best_vals"]), k
    for dg in dgs:
        dg.close()


def test_few_chains_of_a_large_graph_get_eight_warps(rfmf, ctx):
    """32 chains of a 100x200 torus (n = 20000) run eight warps per chain;
    32 chains of ER n = 5000 stay at four (the plan; results do not depend
    on the width)."""
    widths = {}
    for name, g in (("torus", rfmf.torus(100, 200, signed=True, seed=0)),
                    ("er", rfmf.erdos_renyi_sparse(5000, 5, signed=True, seed=0))):
        dg = rfmf.DeviceGraph(ctx, g)
        init, solver = chains_for(g, list(range(32)))
        b = rfmf.Batch(ctx, [dg] * 32, [70.0] * 32, solver, list(init), [8, 1], [4, 4])
        widths[name] = b.info()["threads_per_chain"]
        b.close()
        dg.close()
    assert widths == {"torus": 256, "er": 128}, widths


def test_phase_cuts_with_skipped_and_oversized_phases(rfmf, ctx, oracle):
    """Phase cuts over a schedule with P = 0 phases (skipped, sweep ids not
    advanced) and a P larger than n (the kernel clamps it): a two-graph
    class run in windows that straddle every boundary still equals the
    oracle, chain for chain."""
    graphs = [rfmf.erdos_renyi(240, 0.05, signed=True, seed=21),
              rfmf.torus(12, 20, signed=True, seed=22)]
    phases, iters = [0, 5000, 0, 3, 1], [70, 130, 50, 110, 90]
    dgs = [rfmf.DeviceGraph(ctx, g) for g in graphs]
    gl, ini, sol, t0, per = [], [], [], [], []
    for k, g in enumerate(graphs):
        init, solver = chains_for(g, list(range(40 * k, 40 * k + 24)))
        ts = [40.0 + 20 * (i % 6) for i in range(24)]
        per.append((init, solver, ts))
        gl += [dgs[k]] * 24
        ini += list(init)
        sol += solver
        t0 += ts
    b = rfmf.Batch(ctx, gl, t0, sol, ini, phases, iters)
    assert b.info()["launch_classes"] == 1
    for w in (57, 100, 1000):
        b.run(w)
    r = b.read()
    info = b.info()
    b.close()
    # executed sweeps: 130 (P = 5000) then 110 (P = 3) then 90 (P = 1);
    # windows [0,57) [57,157) [157,330): 1 + 2 + 2 launches
    assert info["launches"] == 5, info
    for k, g in enumerate(graphs):
        init, solver, ts = per[k]
        ref = oracle.anneal(g, init, ts, solver, phases, iters)
        sl = slice(24 * k, 24 * k + 24)
        assert np.array_equal(np.stack(r["end_spins"][sl]), ref["end_spins"]), k
        assert np.array_equal(np.stack(r["best_spins"][sl]), ref["best_spins"]), k
        assert np.array_equal(r["best_vals"][sl], ref["best_vals"]), k
    for dg in dgs:
        dg.close()


def test_chain_width_follows_the_phase(rfmf, ctx, oracle):
    """One dense graph with 700 chains (one warp per chain by rule; every
    chain still resident at two): the P = 128 phase, whose winner rows hold
    more entries than the graph has vertices, runs two warps per chain and
    the later phases one; windows straddle the switches and every chain
    equals the oracle."""
    g = rfmf.erdos_renyi_degree(600, 19, signed=True, seed=8)
    C = 700
    init, solver = chains_for(g, list(range(3000, 3000 + C)))
    t0s = [35.0 + 15 * (i % 8) for i in range(C)]
    phases, iters = [128, 16, 1], [150, 150, 150]
    dg = rfmf.DeviceGraph(ctx, g)
    b = rfmf.Batch(ctx, [dg] * C, t0s, solver, list(init), phases, iters)
    b.run_timed(100)
    wide = b.info()["threads_per_chain"]
    b.run_timed(100)
    narrow = b.info()["threads_per_chain"]
    b.run(1000)
    info = b.info()
    r = b.read()
    b.close()
    dg.close()
    assert (wide, narrow) == (64, 32), (wide, narrow)
    # [0,100) P=128; [100,150) P=128 + [150,200) P=16; [200,300) P=16 + [300,450) P=1
    assert info["launches"] == 5, info
    ref = oracle.anneal(g, init, t0s, solver, phases, iters)
    assert np.array_equal(np.stack(r["end_spins"]), ref["end_spins"])
    assert np.array_equal(np.stack(r["best_spins"]), ref["best_spins"])
    assert np.array_equal(r["cur_vals"], ref["cur_vals"])
    assert np.array_equal(r["best_vals"], ref["best_vals"])


def test_four_warp_chains_widen_to_eight_in_row_heavy_phases(rfmf, ctx, oracle):
    """32 chains of ER n = 800 p = 0.06 (four warps per chain by rule): eight
    warps in the P = 128 phase, four after; every chain equals the oracle."""
    g = rfmf.erdos_renyi(800, 0.06, seed=0)
    C = 32
    init, solver = chains_for(g, list(range(C)))
    t0s = [35.0 + 15 * (i % 8) for i in range(C)]
    phases, iters = [128, 1], [120, 120]
    dg = rfmf.DeviceGraph(ctx, g)
    b = rfmf.Batch(ctx, [dg] * C, t0s, solver, list(init), phases, iters)
    b.run_timed(100)
    wide = b.info()["threads_per_chain"]
    b.run_timed(1000)
    narrow = b.info()["threads_per_chain"]
    r = b.read()
    b.close()
    dg.close()
    assert (wide, narrow) == (256, 128), (wide, narrow)
    ref = oracle.anneal(g, init, t0s, solver, phases, iters)
    assert np.array_equal(np.stack(r["end_spins"]), ref["end_spins"])
    assert np.array_equal(np.stack(r["best_spins"]), ref["best_spins"])
    assert np.array_equal(r["best_vals"], ref["best_vals"])


def test_one_graph_past_one_round_of_ctas(rfmf, ctx, oracle):
    """More one-warp chains of one graph than one round of 16-chain CTAs
    holds (2600 > 16 x 152): the planner sizes the items for the queue's
    list schedule (smaller items than 16); every chain equals the oracle."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    g = rfmf.erdos_renyi(300, 0.04, signed=True, seed=12)
    C = 16 * sms + 168
    init, solver = chains_for(g, list(range(8000, 8000 + C)))
    t0s = [35.0 + 15 * (i % 8) for i in range(C)]
    phases, iters = [32, 1], [100, 100]
    dg = rfmf.DeviceGraph(ctx, g)
    b = rfmf.Batch(ctx, [dg] * C, t0s, solver, list(init), phases, iters)
    assert b.info()["threads_per_chain"] == 32
    b.run(200)
    info = b.info()
    r = b.read()
    b.close()
    dg.close()
    assert info["items"] > -(-C // 16), info
    ref = oracle.anneal(g, init, t0s, solver, phases, iters)
    assert np.array_equal(np.stack(r["end_spins"]), ref["end_spins"])
    assert np.array_equal(np.stack(r["best_spins"]), ref["best_spins"])
    assert np.array_equal(r["best_vals"], ref["best_vals"])
