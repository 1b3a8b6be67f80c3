"""Graph ingest on the device (rfmf_graph_from_edges) and the device output
path (rfmf_batch_cuts, rfmf_batch_partitions).

The device CSR build must give the CSR the reference's loader gives
(digests from tests/golden/ingest_cases.json, produced by the reference's
own code) and graphs that anneal exactly like host-built ones; the device cut
recompute must equal the host's and the kernel's tracked cuts; the partition
strings must equal the spins read back."""
import hashlib
import json
import pathlib

import numpy as np
import pytest

from conftest import chains_for

pytestmark = pytest.mark.gpu
GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
CASES = json.loads((GOLDEN / "ingest_cases.json").read_text())["cases"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_device_csr_matches_reference_loader(rfmf, ctx, case):
    d = rfmf.parse_gset(case["text"])
    dg = rfmf.DeviceGraph.from_edges(ctx, d["u"], d["v"], d["w"])
    off, col, w = dg.csr()
    h = hashlib.sha256(off.tobytes() + col.tobytes() + w.tobytes()).hexdigest()
    info = dg.info()
    assert (dg.n, info["m"], info["max_weighted_degree"], h) == \
        (case["n"], case["m"], case["B"], case["sha256"])
    ids = np.unique(np.concatenate([d["u"], d["v"]]))
    assert np.array_equal(dg.orig_ids(), ids)


def test_device_csr_random_against_host_builder(rfmf, ctx):
    rng = np.random.default_rng(5)
    for trial in range(4):
        E = int(rng.integers(1, 30000))
        ids = rng.choice(200000, size=int(rng.integers(2, 4000)), replace=False)
        u = rng.choice(ids, E)
        v = rng.choice(ids, E)
        keep = u != v
        u, v = u[keep], v[keep]
        w = rng.integers(-3, 4, len(u))
        w[w == 0] = 1
        host = rfmf.csr_from_edges(u, v, w)
        dg = rfmf.DeviceGraph.from_edges(ctx, u, v, w)
        off, col, ww = dg.csr()
        assert dg.n == host.n
        assert np.array_equal(off, host.offsets.astype(np.uint32))
        assert np.array_equal(col, host.col.astype(np.int32))
        assert np.array_equal(ww, host.weight.astype(np.int32))


def test_device_built_graph_anneals_like_host_built(rfmf, ctx):
    g = rfmf.erdos_renyi(500, 0.03, signed=True, seed=17)
    src = np.repeat(np.arange(g.n), np.diff(g.offsets))
    up = g.col > src
    dg_dev = rfmf.DeviceGraph.from_edges(ctx, src[up], g.col[up], g.weight[up])
    dg_host = rfmf.DeviceGraph(ctx, g)
    init, solver = chains_for(g, list(range(24)))
    t0s = [35.0, 100.0, 400.0] * 8
    a = rfmf.anneal_gpu(ctx, dg_dev, g.max_weighted_degree(), init, t0s, [32, 4, 1], [300] * 3, solver)
    b = rfmf.anneal_gpu(ctx, dg_host, g.max_weighted_degree(), init, t0s, [32, 4, 1], [300] * 3, solver)
    assert np.array_equal(a.best_spins, b.best_spins) and np.array_equal(a.end_spins, b.end_spins)
    assert np.array_equal(a.best_vals, b.best_vals)


def test_batch_output_path(rfmf, ctx):
    gs = [rfmf.torus(10, 13, signed=True, seed=2), rfmf.erdos_renyi(333, 0.02, seed=3)]
    dgs = [rfmf.DeviceGraph(ctx, g) for g in gs]
    gl, ini, sol, t0 = [], [], [], []
    for k, g in enumerate(gs):
        init, solver = chains_for(g, list(range(100 * k, 100 * k + 20)))
        gl += [dgs[k]] * 20
        ini += list(init)
        sol += solver
        t0 += [50.0] * 20
    b = rfmf.Batch(ctx, gl, t0, sol, ini, [8, 1], [500, 500])
    b.run(1000)
    r = b.read()
    assert np.array_equal(b.cuts(best=True), r["best_vals"])
    assert np.array_equal(b.cuts(best=False), r["cur_vals"])
    host = [gs[i // 20].cut_value(r["best_spins"][i]) for i in range(40)]
    assert np.array_equal(b.cuts(best=True), host)
    for best in (False, True):
        parts = b.partitions(best=best)
        spins = r["best_spins"] if best else r["end_spins"]
        for p, s in zip(parts, spins):
            assert p == "".join("1" if x > 0 else "0" for x in s)
    b.close()
