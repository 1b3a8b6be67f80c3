#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Run where the reference checkout and oracle/_ref/libref_host.so exist
(oracle/build_ref.sh builds it from the reference's host sources).  Every
value below comes from the reference's host code, never from this project's
library or oracle; the tests then check both against these files.

  philox_kat.json    Philox4x32-10 blocks (src/philox.cuh:89-119) and the
                     Q20 Gumbel of every 11-bit field (src/philox.cuh:52-58)
  beta_tables.json   buildBetaRunTables (src/host_common.cpp:212-294) run
                     counts, digests and edge runs; betaFixedForStep samples
  score_gate.json    annealScoreSafeInt32 verdicts (src/host_common.cpp:296-312)
  initial_spins.json Rng(seed).bits(1) spins (src/rng.hpp, host_common.cpp:40-45)
  gset_csr.json      CSR digests of Gset graphs through the reference loader
                     (src/read_gset.cpp, src/immutable_graph.hpp), plus B
                     (src/host_common.cpp:314-325) and a cut value
                     (src/max_cut.cpp:5-15) -- digests only, no graph data
  anneal_small.json  anneal results of the oracle on seeded synthetic graphs,
                     recorded after the oracle was pinned (regression fixture
                     for the GPU tests; regenerate with --anneal)
"""
import ctypes as ct
import hashlib
import json
import os
import pathlib
import random
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF = pathlib.Path(os.environ.get("RFMF_REFERENCE", "/root/reference"))
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

P, I64, U64 = ct.c_void_p, ct.c_int64, ct.c_uint64


def ref_lib():
    L = ct.CDLL(str(ROOT / "oracle" / "_ref" / "libref_host.so"))
    L.ref_philox_block.argtypes = [U64, U64, U64, P]
    L.ref_gumbel.argtypes = [ct.c_uint32]
    L.ref_gumbel.restype = ct.c_int32
    L.ref_beta_fixed.argtypes = [U64, ct.c_double]
    L.ref_beta_fixed.restype = ct.c_int32
    L.ref_beta_tables.argtypes = [P, I64, I64, P, P, P, I64]
    L.ref_beta_tables.restype = I64
    L.ref_score_safe_int32.argtypes = [I64, ct.c_double, I64]
    L.ref_score_safe_int32.restype = ct.c_int
    L.ref_initial_spins.argtypes = [U64, I64, P]
    L.ref_gset_load.argtypes = [ct.c_char_p]
    L.ref_gset_load.restype = P
    for f in ("ref_gset_n", "ref_gset_m", "ref_gset_max_weighted_degree"):
        getattr(L, f).argtypes = [P]
        getattr(L, f).restype = I64
    L.ref_gset_copy.argtypes = [P, P, P, P]
    L.ref_gset_cut.argtypes = [P, P]
    L.ref_gset_cut.restype = I64
    L.ref_gset_free.argtypes = [P]
    return L


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def ref_beta(L, t0s, total):
    t = np.array(t0s, np.float64)
    off = np.zeros(len(t), np.int64)
    R = L.ref_beta_tables(t.ctypes.data, len(t), total, None, None, off.ctypes.data, 0)
    e = np.zeros(R, np.int64)
    v = np.zeros(R, np.int32)
    L.ref_beta_tables(t.ctypes.data, len(t), total, e.ctypes.data, v.ctypes.data, off.ctypes.data, R)
    return e, v, off


def make_primitives(L):
    rnd = random.Random(20261203)
    kat = []
    for _ in range(256):
        seed = rnd.getrandbits(64)
        step = rnd.choice([1, 2, 3, rnd.getrandbits(20), rnd.getrandbits(40), rnd.getrandbits(64)])
        block = rnd.choice([0, 1, rnd.getrandbits(12), rnd.getrandbits(33)])
        out = np.zeros(4, np.uint32)
        L.ref_philox_block(seed, step, block, out.ctypes.data)
        kat.append(dict(seed=seed, step=step, block=block, out=[int(x) for x in out]))
    gumbel = [int(L.ref_gumbel(r)) for r in range(2048)]
    (HERE / "philox_kat.json").write_text(json.dumps(dict(blocks=kat, gumbel_by_field=gumbel)) + "\n")

    tables = []
    cases = [([35.0, 50.0, 70.0, 100.0, 140.0, 200.0, 280.0, 400.0], 10**7),
             ([35.0, 50.0, 70.0, 100.0, 140.0, 200.0, 280.0, 400.0], 10**6),
             ([105.0, 90.0, 105.0, 120.0], 1050), ([0.01, 105.0], 300), ([0.5], 20000),
             ([400.0], 0), ([35.0], 1), ([0.002], 50), ([35.0, 400.0], 10**8)]
    for t0s, total in cases:
        e, v, off = ref_beta(L, t0s, total)
        tables.append(dict(t0s=t0s, total=total, runs=len(e), chain_off=[int(x) for x in off],
                           sha256=sha(e, v), head=[[int(a), int(b)] for a, b in zip(e[:6], v[:6])],
                           tail=[[int(a), int(b)] for a, b in zip(e[-6:], v[-6:])]))
    steps = [1, 2, 3, 10, 99, 1000, 65535, 10**6, 10**7, 10**9, 10**12]
    samples = [dict(step=s, t0=t, beta=int(L.ref_beta_fixed(s, t)))
               for s in steps for t in (0.01, 0.5, 35.0, 105.0, 400.0)
               if L.ref_beta_fixed(s, t) >= 0]
    (HERE / "beta_tables.json").write_text(json.dumps(dict(tables=tables, samples=samples)) + "\n")

    gate = []
    for T in [0, 1, 100, 10**4, 10**6, 10**7, 10**8, 10**10, 10**12]:
        for t0 in [0.001, 0.01, 0.5, 3.0, 35.0, 400.0]:
            for B in [0, 1, 4, 19, 36, 127, 1000, 10**5, 10**6, 2**31 - 1]:
                gate.append([T, t0, B, int(L.ref_score_safe_int32(T, t0, B))])
    (HERE / "score_gate.json").write_text(json.dumps(dict(cases=gate)) + "\n")

    spins = []
    for seed in [0, 1, 2, 42, 501, 2955857184, 2**63, 2**64 - 1]:
        for n in [1, 63, 64, 65, 800]:
            out = np.zeros(n, np.int8)
            L.ref_initial_spins(seed, n, out.ctypes.data)
            spins.append(dict(seed=seed, n=n, bits="".join("1" if s > 0 else "0" for s in out)))
    (HERE / "initial_spins.json").write_text(json.dumps(dict(cases=spins)) + "\n")


def make_gset(L):
    out = []
    for name in ["G1", "G11", "G14", "G22", "G43", "G48", "G55", "G60", "G62", "G63", "G70",
                 "G81"]:
        path = REF / "Gset" / name
        if not path.exists():
            continue
        h = L.ref_gset_load(str(path).encode())
        n, m = L.ref_gset_n(h), L.ref_gset_m(h)
        off = np.zeros(n + 1, np.uint32)
        col = np.zeros(2 * m, np.int32)
        w = np.zeros(2 * m, np.int32)
        L.ref_gset_copy(h, off.ctypes.data, col.ctypes.data, w.ctypes.data)
        spin = np.zeros(n, np.int8)
        L.ref_initial_spins(7, n, spin.ctypes.data)
        out.append(dict(name=name, n=n, m=m, B=int(L.ref_gset_max_weighted_degree(h)),
                        sha256=sha(off, col, w), cut_seed7=int(L.ref_gset_cut(h, spin.ctypes.data))))
        L.ref_gset_free(h)
    (HERE / "gset_csr.json").write_text(json.dumps(dict(graphs=out), indent=0) + "\n")


ANNEAL_CASES = [
    dict(graph=("erdos_renyi", dict(n=800, p=0.06, seed=0)), seeds=list(range(8)),
         t0s=[35.0, 50.0, 70.0, 100.0, 140.0, 200.0, 280.0, 400.0],
         phases=[128, 64, 32, 16, 8, 4, 2, 1], iters=[300] * 8),
    dict(graph=("torus", dict(rows=20, cols=30, signed=True, seed=1)), seeds=[1, 2, 3],
         t0s=[105.0, 90.0, 105.0], phases=[64, 32, 16, 8, 4, 2, 1], iters=[120] * 7),
    dict(graph=("erdos_renyi", dict(n=200, p=0.05, seed=12)), seeds=[42, 42],
         t0s=[0.01, 105.0], phases=[8, 4], iters=[150, 150]),
    dict(graph=("random_tree", dict(n=500, signed=True, seed=3)), seeds=[13, 14],
         t0s=[105.0, 105.0], phases=[8, 2, 1], iters=[150, 150, 150]),
    dict(graph=("planar_like", dict(n=400, seed=4)), seeds=[5, 6, 7],
         t0s=[35.0, 100.0, 400.0], phases=[100, 7, 3, 1], iters=[90, 90, 90, 90]),
]


def partition_sha(spins):
    return hashlib.sha256("".join("0" if s < 0 else "1" for s in spins).encode()).hexdigest()


def make_anneal():
    import oracle as ora
    import rfmf_gb300.graphs as G
    out = []
    for case in ANNEAL_CASES:
        fn, kw = case["graph"]
        g = getattr(G, fn)(**kw)
        init = np.stack([ora.initial_spins(s, g.n) for s in case["seeds"]])
        solver = [(s + 0xC2B2AE3D27D4EB4F) % 2**64 for s in case["seeds"]]
        r = ora.anneal(g, init, case["t0s"], solver, case["phases"], case["iters"])
        out.append(dict(case, graph=[fn, kw], n=g.n, m=g.m, csr_sha256=sha(g.offsets, g.col, g.weight),
                        best=[int(x) for x in r["best_vals"]], final=[int(x) for x in r["cur_vals"]],
                        best_partition_sha256=[partition_sha(x) for x in r["best_spins"]],
                        final_partition_sha256=[partition_sha(x) for x in r["end_spins"]]))
    (HERE / "anneal_small.json").write_text(json.dumps(dict(cases=out), indent=0) + "\n")


if __name__ == "__main__":
    if "--anneal" in sys.argv:
        make_anneal()
    else:
        L = ref_lib()
        make_primitives(L)
        make_gset(L)
        make_anneal()
    print("golden fixtures written to", HERE)
