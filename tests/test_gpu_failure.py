"""Failure detection on the device, driven from the host.

The kernel checks, at the start of every launch window, that each chain's
carried cut equals the cut recomputed from its spins; an inconsistency sets
the launch's device error word (no trap, no wait) and the batch reports
RFMF_ERR_DEVICE.  The inconsistency is planted from the host with the
library's testing aid (a chain's carried cut overwritten between windows);
afterwards the same context must still run batches correctly."""
import numpy as np
import pytest

from conftest import chains_for

pytestmark = pytest.mark.gpu


def _batch(rfmf, ctx, dg, g, seeds, phases, iters):
    init, solver = chains_for(g, seeds)
    return rfmf.Batch(ctx, [dg] * len(seeds), [70.0] * len(seeds), solver, list(init), phases, iters)


def test_device_error_reported_and_context_usable(rfmf, ctx):
    g = rfmf.erdos_renyi(300, 0.05, signed=True, seed=21)
    dg = rfmf.DeviceGraph(ctx, g)
    phases, iters = [16, 1], [200, 200]
    b = _batch(rfmf, ctx, dg, g, [1, 2, 3, 4], phases, iters)
    b.run(100)
    b.synchronize()
    cur = b.read()["cur_vals"]
    b.debug_set_cut(2, int(cur[2]) + 1)
    with pytest.raises(rfmf.RfmfError) as err:
        b.run(100)
        b.synchronize()
    assert "RFMF_ERR_DEVICE" in str(err.value), str(err.value)
    b.close()

    # The context is still usable: a fresh batch equals the synchronous
    # drop-in on the same inputs.
    seeds = [5, 6, 7]
    init, solver = chains_for(g, seeds)
    fresh = rfmf.Batch(ctx, [dg] * 3, [70.0] * 3, solver, list(init), phases, iters)
    fresh.run(sum(iters))
    out = fresh.read()
    fresh.close()
    ref = rfmf.anneal_gpu(ctx, dg, g.max_weighted_degree(), init, [70.0] * 3, phases, iters, solver)
    assert np.array_equal(np.stack(out["end_spins"]), ref.end_spins)
    assert np.array_equal(np.asarray(out["best_vals"]), ref.best_vals)


def test_debug_set_cut_rejects_bad_chain(rfmf, ctx):
    g = rfmf.torus(6, 7, signed=True, seed=3)
    dg = rfmf.DeviceGraph(ctx, g)
    b = _batch(rfmf, ctx, dg, g, [1, 2], [4, 1], [10, 10])
    with pytest.raises(rfmf.RfmfError):
        b.debug_set_cut(5, 0)
    b.close()
