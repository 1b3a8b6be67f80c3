"""Host input path: CSR canonicalisation, the Gset reader, and the seeded
synthetic generators of the benchmark shapes."""
import hashlib
import json

import numpy as np
import pytest

from conftest import GOLDEN, REFERENCE


def check_canonical(g):
    off = g.offsets.astype(np.int64)
    assert off[0] == 0 and np.all(np.diff(off) >= 0) and off[-1] == len(g.col)
    src = np.repeat(np.arange(g.n), np.diff(off))
    assert np.all(g.col != src)                                  # no self loops
    for v in range(g.n):                                         # rows strictly ascending
        row = g.col[off[v]:off[v + 1]]
        assert np.all(np.diff(row) > 0)
    fwd = {(int(a), int(b)): int(w) for a, b, w in zip(src, g.col, g.weight)}
    assert all(fwd[(b, a)] == w for (a, b), w in fwd.items())    # symmetric
    assert np.all(np.diff(off) > 0)                              # no isolated vertices


def test_csr_from_edges_semantics(rfmf):
    # duplicates keep the FIRST weight (Graph::addEdge), self loops dropped,
    # isolated ids never appear, ids renumbered by ascending original id
    g = rfmf.csr_from_edges([10, 3, 10, 7, 7], [3, 10, 20, 7, 3], [5, 9, -2, 4, 1])
    assert g.n == 4 and list(g.orig_ids) == [3, 7, 10, 20]
    check_canonical(g)
    w = {(int(a), int(b)): int(x) for a, b, x in
         zip(np.repeat(np.arange(g.n), np.diff(g.offsets.astype(np.int64))), g.col, g.weight)}
    assert w[(0, 2)] == 5 and w[(2, 3)] == -2 and w[(0, 1)] == 1


@pytest.mark.parametrize("make", [
    lambda R: R.erdos_renyi(800, 0.06, seed=0),
    lambda R: R.torus(50, 60, signed=True, seed=0),
    lambda R: R.erdos_renyi_degree(2000, 19, signed=True, seed=0),
    lambda R: R.random_tree(1000, seed=0),
    lambda R: R.planar_like(800, seed=0),
])
def test_generators_canonical(rfmf, make):
    check_canonical(make(rfmf))


def test_benchmark_shapes(rfmf):
    er = rfmf.erdos_renyi(800, 0.06, seed=0)
    assert er.n == 800 and abs(er.m - 19176) < 600 and set(np.unique(er.weight)) == {1}
    t = rfmf.torus(50, 60, signed=True, seed=0)
    assert t.n == 3000 and t.m == 6000 and t.max_weighted_degree() == 4
    assert set(np.unique(t.weight)) == {-1, 1}
    e2 = rfmf.erdos_renyi_degree(2000, 19, signed=True, seed=0)
    assert e2.n == 2000 and abs(2 * e2.m / e2.n - 19) < 0.5
    tr = rfmf.random_tree(10000, seed=0)
    assert tr.n == 10000 and tr.m == 9999
    big = rfmf.torus(100, 200, signed=True, seed=0)
    assert big.n == 20000 and big.m == 40000
    pl = rfmf.planar_like(2000, seed=0)
    assert abs(2 * pl.m / pl.n - 11.7) < 1.0


def test_generators_deterministic(rfmf):
    a = rfmf.erdos_renyi_degree(500, 7, signed=True, seed=3)
    b = rfmf.erdos_renyi_degree(500, 7, signed=True, seed=3)
    assert np.array_equal(a.col, b.col) and np.array_equal(a.weight, b.weight)


def test_gset_reader_matches_reference_loader(rfmf):
    """The Python Gset reader builds the same CSR as the reference's loader
    (digests recorded from src/read_gset.cpp + src/immutable_graph.hpp)."""
    recs = json.loads((GOLDEN / "gset_csr.json").read_text())["graphs"]
    if not (REFERENCE / "Gset").exists():
        pytest.skip("Gset files not present")
    for r in recs[:6]:
        g = rfmf.read_gset(REFERENCE / "Gset" / r["name"])
        h = hashlib.sha256(g.offsets.tobytes() + g.col.tobytes() + g.weight.tobytes()).hexdigest()
        assert (g.n, g.m, h) == (r["n"], r["m"], r["sha256"]), r["name"]
        assert g.max_weighted_degree() == r["B"]
        assert g.cut_value(rfmf.initial_spins(7, g.n)) == r["cut_seed7"]
