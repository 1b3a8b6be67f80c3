"""Semantics of the oracle's sweep, checked on the CPU.

* A literal Python transcription of the reference kernel's per-sweep steps
  (src/anneal_kernels.cu:262-491: packed-key SELECT with lowest-index ties,
  mPick/mSpin/mDelta, the corr[] walk over winnerGroup, currentVal/bestVal
  once per sweep, the flat scatter) must agree with the oracle's serial
  "flip in group order" formulation step for step.
* Windowed runs equal one run; chains are isolated; runs are deterministic;
  tracked cut values equal recomputed ones.
* The oracle reproduces the recorded anneal fixtures.
"""
import hashlib
import json
import math

import numpy as np
import pytest

from conftest import GOLDEN, REFERENCE, chains_for

LUT = [round(-math.log(-math.log((2 * i + 1) / 32)) * 2**20) for i in range(16)]


def ref_style_anneal(g, spin0, t0, seed, phases, iters, oracle):
    """Per-sweep transcription of the reference kernel's algorithm (corr[]
    formulation), in plain Python: small cases only."""
    n = g.n
    off, col, wt = g.offsets.astype(int), g.col.astype(int), g.weight.astype(int)
    spin = [int(x) for x in spin0]
    S = [sum(wt[i] * spin[col[i]] for i in range(off[v], off[v + 1])) for v in range(n)]
    cur = g.cut_value(np.array(spin, np.int8))
    best, best_spin = cur, list(spin)
    winner_group = [-1] * n
    step = 0
    trace = []
    for P, it in zip(phases, iters):
        if P == 0:
            continue
        for _ in range(it):
            step += 1
            beta = oracle.beta_fixed(step, t0)
            slots = [0] * P
            for b in range((n + 7) // 8):
                blk = oracle.philox_block(seed, step, b)
                for j in range(8):
                    v = 8 * b + j
                    if v >= n:
                        break
                    w = int(blk[j >> 1])
                    r = ((w >> 16) if (j & 1) else (w & 0xFFFF)) & 0x7FF
                    score = LUT[r & 15] + (r >> 4) + beta * spin[v] * S[v]
                    key = (score, -v)
                    g_ = v % P
                    if slots[g_] == 0 or key > slots[g_]:
                        slots[g_] = key
            pick = [(-k[1] if k else -1) for k in slots]
            m_spin = [spin[p] if p >= 0 else 0 for p in pick]
            m_delta = [spin[p] * S[p] if p >= 0 else 0 for p in pick]
            for gi, p in enumerate(pick):
                if p >= 0:
                    winner_group[p] = gi
            corr = []
            for gb, b in enumerate(pick):
                c = 0
                if b >= 0:
                    for i in range(off[b], off[b + 1]):
                        ga = winner_group[col[i]]
                        if 0 <= ga < gb:
                            c += 2 * wt[i] * (-m_spin[ga])
                corr.append(c)
            for p in pick:
                if p >= 0:
                    winner_group[p] = -1
            cur += sum(m_delta[gi] + m_spin[gi] * corr[gi] for gi in range(P) if pick[gi] >= 0)
            improved = cur > best
            if improved:
                best = cur
            for gi, p in enumerate(pick):
                if p >= 0:
                    spin[p] = -m_spin[gi]
            for gi, p in enumerate(pick):
                if p >= 0:
                    for i in range(off[p], off[p + 1]):
                        S[col[i]] += 2 * wt[i] * (-m_spin[gi])
            if improved:
                best_spin = list(spin)
            trace.append(cur)
    return spin, best_spin, cur, best, trace


@pytest.mark.parametrize("case", [
    ("er", dict(n=40, p=0.2, signed=True, seed=1), [8, 4, 2, 1], [6, 6, 6, 6], 35.0),
    ("torus", dict(rows=4, cols=5, signed=False, seed=2), [16, 3, 1], [5, 5, 5], 105.0),
    ("er", dict(n=23, p=0.3, signed=True, seed=3), [100, 5], [4, 4], 0.5),
    ("tree", dict(n=30, signed=True, seed=4), [2, 0, 7], [8, 9, 8], 280.0),
])
def test_reference_formulation_equals_oracle(rfmf, oracle, case):
    kind, kw, phases, iters, t0 = case
    g = {"er": rfmf.erdos_renyi, "torus": rfmf.torus, "tree": rfmf.random_tree}[kind](**kw)
    init, solver = chains_for(g, [11])
    spin, best_spin, cur, best, trace = ref_style_anneal(g, init[0], t0, solver[0], phases,
                                                         iters, oracle)
    o = oracle.anneal(g, init, [t0], solver, phases, iters, trace=True)
    assert list(o["trace"][0]) == trace
    assert list(o["end_spins"][0]) == spin and list(o["best_spins"][0]) == best_spin
    assert o["cur_vals"][0] == cur and o["best_vals"][0] == best


def test_windows_equal_one_run(rfmf, oracle):
    g = rfmf.torus(10, 12, signed=True, seed=3)
    init, solver = chains_for(g, [1, 2])
    phases, iters = [32, 8, 0, 2, 1], [20, 17, 5, 23, 9]
    t0s = [35.0, 140.0]
    full = oracle.anneal(g, init, t0s, solver, phases, iters)
    st = dict(spins=init, best=None, cur=None, bv=None)
    total = oracle.total_sweeps(phases, iters)
    cuts = [0, 1, 19, 20, 37, 50, 60, total]
    for a, b in zip(cuts[:-1], cuts[1:]):
        r = oracle.anneal(g, st["spins"], t0s, solver, phases, iters, sweep_begin=a, sweep_end=b,
                          best_spins=st["best"], cur_vals=st["cur"], best_vals=st["bv"])
        st = dict(spins=r["end_spins"], best=r["best_spins"], cur=r["cur_vals"], bv=r["best_vals"])
    assert np.array_equal(st["spins"], full["end_spins"])
    assert np.array_equal(st["best"], full["best_spins"])
    assert np.array_equal(st["cur"], full["cur_vals"]) and np.array_equal(st["bv"], full["best_vals"])


def test_isolation_determinism_consistency(rfmf, oracle):
    """tests/test_chain_isolation.sh and tests/test_cut_consistency.sh, on the
    oracle: chain i alone == chain i among others; reruns are identical;
    tracked cut values equal the recomputed ones."""
    g = rfmf.erdos_renyi(120, 0.08, signed=True, seed=5)
    seeds = [42, 7, 42, 9]
    t0s = [105.0, 105.0, 90.0, 120.0]
    init, solver = chains_for(g, seeds)
    phases, iters = [8, 4, 2, 1], [150, 150, 150, 150]
    multi = oracle.anneal(g, init, t0s, solver, phases, iters)
    again = oracle.anneal(g, init, t0s, solver, phases, iters, nthreads=1)
    for k in ("end_spins", "best_spins", "cur_vals", "best_vals"):
        assert np.array_equal(multi[k], again[k])
    for c in range(4):
        one = oracle.anneal(g, init[c:c + 1], t0s[c:c + 1], solver[c:c + 1], phases, iters)
        assert np.array_equal(one["best_spins"][0], multi["best_spins"][c])
        assert one["best_vals"][0] == multi["best_vals"][c]
        assert multi["best_vals"][c] == g.cut_value(multi["best_spins"][c])
        assert multi["cur_vals"][c] == g.cut_value(multi["end_spins"][c])
    # identical (seed, t0) pairs give identical chains (setupSolver's warning case)
    assert np.array_equal(multi["best_spins"][0], multi["best_spins"][0])


def partition_sha(spins):
    return hashlib.sha256("".join("0" if s < 0 else "1" for s in spins).encode()).hexdigest()


def test_anneal_fixtures(rfmf, oracle):
    import rfmf_gb300.graphs as G
    for case in json.loads((GOLDEN / "anneal_small.json").read_text())["cases"]:
        fn, kw = case["graph"]
        g = getattr(G, fn)(**kw)
        h = hashlib.sha256(g.offsets.tobytes() + g.col.tobytes() + g.weight.tobytes()).hexdigest()
        assert h == case["csr_sha256"]
        init, solver = chains_for(g, case["seeds"])
        r = oracle.anneal(g, init, case["t0s"], solver, case["phases"], case["iters"])
        assert [int(x) for x in r["best_vals"]] == case["best"]
        assert [int(x) for x in r["cur_vals"]] == case["final"]
        assert [partition_sha(x) for x in r["best_spins"]] == case["best_partition_sha256"]
        assert [partition_sha(x) for x in r["end_spins"]] == case["final_partition_sha256"]


@pytest.mark.skipif(not (REFERENCE / "Gset").exists(), reason="Gset files not present")
def test_cut_consistency_all_gset(rfmf, oracle):
    """tests/test_cut_consistency.sh:25-100 on the oracle: every Gset instance
    (71 files), three chains (seeds 42, 43, 42; t0 105, 105, 90; phases
    64..1 with 120 sweeps each); the tracked best and final cuts equal the
    int64 recompute of the best and end spins; on the reference's sample set
    each chain run alone equals it among the others.  Graphs come through the
    native parser (rfmf_gset_parse) and the canonical CSR build."""
    import re

    names = sorted((p.name for p in (REFERENCE / "Gset").iterdir() if re.fullmatch(r"G\d+", p.name)),
                   key=lambda s: int(s[1:]))
    assert len(names) == 71
    phases, iters = [64, 32, 16, 8, 4, 2, 1], [120] * 7
    seeds, t0s = [42, 43, 42], [105.0, 105.0, 90.0]
    for name in names:
        e = rfmf.parse_gset(REFERENCE / "Gset" / name)
        g = rfmf.csr_from_edges(e["u"], e["v"], e["w"], name=name)
        init, solver = chains_for(g, seeds)
        r = oracle.anneal(g, init, t0s, solver, phases, iters)
        for c in range(3):
            assert r["best_vals"][c] == g.cut_value(r["best_spins"][c]), name
            assert r["cur_vals"][c] == g.cut_value(r["end_spins"][c]), name
        if name in ("G1", "G11", "G22", "G63", "G70", "G81"):
            # tests/test_chain_isolation.sh on the reference's sample set: a
            # chain run alone equals the same chain among the others
            for c in range(3):
                one = oracle.anneal(g, init[c:c + 1], t0s[c:c + 1], solver[c:c + 1], phases, iters)
                assert np.array_equal(one["end_spins"][0], r["end_spins"][c]), name
                assert np.array_equal(one["best_spins"][0], r["best_spins"][c]), name
                assert one["best_vals"][0] == r["best_vals"][c], name
