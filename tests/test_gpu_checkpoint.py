"""Checkpoint and resume: what rfmf_batch_read returns is a checkpoint, and
rfmf_batch_restore (in the same or a new context) resumes it.  A chain is a
pure function of (graph, seed, t0, schedule, sweep index)
(src/anneal_gpu.cuh:4-8), so an anneal split into pieces at any sweep and
resumed from host state must equal one uninterrupted run bit for bit."""
import numpy as np
import pytest

from conftest import chains_for

pytestmark = pytest.mark.gpu

PHASES = [64, 16, 4, 1]
ITERS = [300, 300, 300, 300]


def _setup(rfmf, ctx):
    graphs = [rfmf.erdos_renyi(600, 0.03, signed=True, seed=41),
              rfmf.torus(20, 30, signed=True, seed=42)]
    dgs, gl, init, solver, t0s = [], [], [], [], []
    for k, g in enumerate(graphs):
        dg = rfmf.DeviceGraph(ctx, g)
        dgs.append(dg)
        seeds = list(range(100 * k, 100 * k + 24))
        i, s = chains_for(g, seeds)
        gl += [dg] * 24
        init += list(i)
        solver += s
        t0s += [35.0, 70.0, 140.0, 280.0] * 6
    return graphs, dgs, gl, init, solver, t0s


def _same_state(a, b):
    for key in ("cur_vals", "best_vals", "sweeps_done"):
        assert np.array_equal(a[key], b[key]), key
    for key in ("end_spins", "best_spins"):
        assert all(np.array_equal(x, y) for x, y in zip(a[key], b[key])), key


def test_restore_equals_uninterrupted_run(rfmf, ctx):
    graphs, dgs, gl, init, solver, t0s = _setup(rfmf, ctx)
    full = rfmf.Batch(ctx, gl, t0s, solver, init, PHASES, ITERS)
    full.run(sum(ITERS))
    want = full.read()
    full.close()
    # pieces of 333, 1, 500 and the rest sweeps, each resumed from host state,
    # the second piece in a fresh context (as another process would)
    state = None
    for k, piece in enumerate([333, 1, 500, sum(ITERS)]):
        c = rfmf.Context(0) if k == 1 else ctx
        mine = [rfmf.DeviceGraph(c, g) for g in graphs] if k == 1 else dgs
        gl_k = [mine[0]] * 24 + [mine[1]] * 24
        if state is None:
            b = rfmf.Batch(c, gl_k, t0s, solver, init, PHASES, ITERS)
        else:
            b = rfmf.Batch.restore(c, gl_k, t0s, solver, PHASES, ITERS, state)
        b.run(piece)
        state = b.read()
        b.close()
        if k == 1:
            for d in mine:
                d.close()
            c.close()
    _same_state(state, want)


def test_restore_refuses_inconsistent_checkpoint(rfmf, ctx):
    graphs, dgs, gl, init, solver, t0s = _setup(rfmf, ctx)
    b = rfmf.Batch(ctx, gl, t0s, solver, init, PHASES, ITERS)
    b.run(200)
    state = b.read()
    b.close()
    bad = dict(state, cur_vals=state["cur_vals"].copy())
    bad["cur_vals"][5] += 1
    with pytest.raises(rfmf.RfmfError) as ei:
        rfmf.Batch.restore(ctx, gl, t0s, solver, PHASES, ITERS, bad)
    assert ei.value.code == 1
    bad = dict(state, best_vals=state["best_vals"].copy())
    bad["best_vals"][30] -= 2
    with pytest.raises(rfmf.RfmfError):
        rfmf.Batch.restore(ctx, gl, t0s, solver, PHASES, ITERS, bad)
    bad = dict(state, sweeps_done=state["sweeps_done"].copy())
    bad["sweeps_done"][0] = sum(ITERS) + 1
    with pytest.raises(rfmf.RfmfError):
        rfmf.Batch.restore(ctx, gl, t0s, solver, PHASES, ITERS, bad)
    # the consistent checkpoint still resumes
    r = rfmf.Batch.restore(ctx, gl, t0s, solver, PHASES, ITERS, state)
    r.run(sum(ITERS))
    assert all(int(d) == sum(ITERS) for d in r.read()["sweeps_done"])
    r.close()
