"""Measured launch planning (rfmf_autotune): on the benchmark configurations'
shapes, the plan the tuner picks is within 5% of the fastest candidate when
every candidate is timed again, the choice is cached per batch shape, and a
batch run with the tuned plan gives the same results as the default plan
(every plan is output-invariant).  The reference's plan is a fixed V100
table (src/tuning.hpp:10-17)."""
import numpy as np
import pytest

from conftest import chains_for

pytestmark = pytest.mark.gpu

LADDER = [35.0, 50.0, 70.0, 100.0, 140.0, 200.0, 280.0, 400.0]
PHASES = [128, 64, 32, 16, 8, 4, 2, 1]


def _shape(rfmf, ctx, name):
    if name == "mid":
        graphs, C = [rfmf.torus(50, 60, signed=True, seed=0),
                     rfmf.erdos_renyi_degree(2000, 19, signed=True, seed=0)], 1024
    elif name == "large_sparse":
        graphs, C = [rfmf.torus(100, 200, signed=True, seed=0), rfmf.random_tree(10000, seed=0),
                     rfmf.erdos_renyi_sparse(5000, 5, signed=True, seed=0)], 256
    else:
        rng = np.random.default_rng(3)
        graphs, C = [], 64
        for i in range(24):
            n = int(np.exp(rng.uniform(np.log(800), np.log(20000))))
            d, r = float(rng.uniform(5, 48)), max(3, int(n ** 0.5))
            if i % 3 == 0:
                graphs.append(rfmf.erdos_renyi_sparse(n, d, signed=bool(i % 2), seed=100 + i))
            elif i % 3 == 1:
                graphs.append(rfmf.torus(r, max(3, n // r), signed=bool(i % 2), seed=100 + i))
            else:
                graphs.append(rfmf.planar_like(n, 11.7, signed=bool(i % 2), seed=100 + i))
    dgs, gl, init, solver, t0s = [], [], [], [], []
    for k, g in enumerate(graphs):
        dg = rfmf.DeviceGraph(ctx, g)
        dgs.append(dg)
        i, s = chains_for(g, list(range(10000 * k, 10000 * k + C)))
        gl += [dg] * C
        init += list(i)
        solver += s
        t0s += [LADDER[c % 8] for c in range(C)]
    return dgs, gl, init, solver, t0s


def _time(rfmf, ctx, gl, init, solver, t0s, iters, cfg, reps=3):
    """A plan's time on the trial schedule, the way the tuner takes it: one
    untimed run teaches the plan the graphs' costs, then fresh batches are
    timed (median of reps)."""
    b = rfmf.Batch(ctx, gl, t0s, solver, init, PHASES, iters, cfg)
    b.run_timed(sum(iters))
    b.close()
    ts = []
    for _ in range(reps):
        b = rfmf.Batch(ctx, gl, t0s, solver, init, PHASES, iters, cfg)
        ts.append(b.run_timed(sum(iters)))
        b.close()
    return float(np.median(ts))


@pytest.mark.parametrize("name", ["mid", "large_sparse", "mix"])
def test_tuned_plan_is_near_the_fastest_candidate(rfmf, ctx, name):
    dgs, gl, init, solver, t0s = _shape(rfmf, ctx, name)
    iters = [64] * 8                      # the tuner compresses these to 512 sweeps
    best, cands = rfmf.autotune(ctx, gl, t0s, solver, init, PHASES, iters, trial_sweeps=512)
    assert len(cands) == 8
    runnable = [(c, us) for c, us in cands if us >= 0]
    assert runnable
    # the same call again comes from the cache
    best2, cands2 = rfmf.autotune(ctx, gl, t0s, solver, init, PHASES, iters, trial_sweeps=512)
    assert (best2.threads_per_chain, best2.csr_format) == (best.threads_per_chain, best.csr_format)
    assert [us for _, us in cands2] == [us for _, us in cands]
    # every runnable candidate timed again on the same sweeps
    again = [_time(rfmf, ctx, gl, init, solver, t0s, iters, c) for c, _ in runnable]
    mine = _time(rfmf, ctx, gl, init, solver, t0s, iters, best)
    assert mine <= 1.05 * min(again), (name, mine, again)
    # output-invariant: tuned plan vs default plan
    outs = []
    for cfg in (best, rfmf.make_config()):
        b = rfmf.Batch(ctx, gl, t0s, solver, init, PHASES, [16] * 8, cfg)
        b.run(128)
        outs.append(b.read())
        b.close()
    assert np.array_equal(outs[0]["best_vals"], outs[1]["best_vals"])
    assert all(np.array_equal(x, y) for x, y in zip(outs[0]["end_spins"], outs[1]["end_spins"]))
    for d in dgs:
        d.close()
