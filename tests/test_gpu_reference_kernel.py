"""Live comparison with the reference's own GPU kernel, where its cubin
(oracle/_ref/anneal_kernels.cubin, built from the reference's sources by
oracle/build_ref.sh) is present: same inputs, bit-identical outputs."""
import numpy as np
import pytest

from conftest import chains_for

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", ["er", "torus", "tree", "int64"])
def test_live_reference_kernel(rfmf, ctx, refgpu, shape):
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    if shape == "er":
        g, seeds, t0s, ph, it = (rfmf.erdos_renyi(600, 0.03, signed=True, seed=21), list(range(40)),
                                 [35.0 + 10 * i for i in range(40)], [128, 32, 8, 1], [300] * 4)
    elif shape == "torus":
        g, seeds, t0s, ph, it = (rfmf.torus(30, 40, signed=True, seed=22), list(range(170)),
                                 [50.0] * 170, [64, 16, 4, 1], [200] * 4)
    elif shape == "tree":
        g, seeds, t0s, ph, it = (rfmf.random_tree(3000, seed=23), [5, 6], [105.0, 90.0],
                                 [256, 1], [300, 300])
    else:
        g, seeds, t0s, ph, it = (rfmf.erdos_renyi(300, 0.04, seed=24), [1, 2, 3],
                                 [0.01, 0.02, 105.0], [16, 2], [100, 100])
    init, solver = chains_for(g, seeds)
    ref = refgpu.run(g, init, t0s, solver, ph, it, sms)
    dg = rfmf.DeviceGraph(ctx, g)
    res = rfmf.anneal_gpu(ctx, dg, g.max_weighted_degree(), init, t0s, ph, it, solver)
    assert np.array_equal(res.end_spins, ref["end_spins"])
    assert np.array_equal(res.best_spins, ref["best_spins"])
    assert np.array_equal(res.final_vals, ref["cur_vals"])
    assert np.array_equal(res.best_vals, ref["best_vals"])
