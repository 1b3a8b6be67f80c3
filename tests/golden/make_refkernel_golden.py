#!/usr/bin/env python3
"""Golden runs of the REFERENCE's own GPU kernel, recorded as fixtures.

Run on a GPU machine where oracle/_ref/anneal_kernels.cubin exists (built by
oracle/build_ref.sh from the reference's src/anneal_kernels.cu).  For every
case it launches the reference's mcKernel through oracle/refgpu.py with the
reference's own launch choices, checks that the oracle reproduces the result
exactly (pinning the oracle against the reference kernel), and writes the
cut values and partition digests to tests/golden/refkernel_runs.json.  The
GPU tests then require librfmf.so to reproduce those fixtures bit for bit.
"""
import hashlib
import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

LADDER = [35.0, 50.0, 70.0, 100.0, 140.0, 200.0, 280.0, 400.0]
FULL = [128, 64, 32, 16, 8, 4, 2, 1]

CASES = [
    dict(name="er800_p0.06_config1", graph=("erdos_renyi", dict(n=800, p=0.06, seed=0)),
         seeds=list(range(32)), t0s=[LADDER[i % 8] for i in range(32)], phases=FULL,
         iters=[2000] * 8),
    dict(name="torus50x60_pm1", graph=("torus", dict(rows=50, cols=60, signed=True, seed=0)),
         seeds=list(range(64)), t0s=[LADDER[i % 8] for i in range(64)], phases=FULL,
         iters=[1000] * 8),
    dict(name="er2000_d19_pm1_waves", graph=("erdos_renyi_degree", dict(n=2000, avg_degree=19, signed=True, seed=0)),
         seeds=list(range(200)), t0s=[LADDER[i % 8] for i in range(200)], phases=FULL,
         iters=[300] * 8),
    dict(name="tree2000", graph=("random_tree", dict(n=2000, seed=3)), seeds=[13, 14, 15, 16],
         t0s=[105.0, 105.0, 35.0, 400.0], phases=[8, 2, 1], iters=[500, 500, 500]),
    dict(name="int64_path", graph=("erdos_renyi", dict(n=200, p=0.05, seed=12)), seeds=[42, 42],
         t0s=[0.01, 105.0], phases=[8, 4], iters=[150, 150]),
    dict(name="odd_P", graph=("torus", dict(rows=12, cols=17, signed=True, seed=2)),
         seeds=[1, 2, 3], t0s=[70.0, 140.0, 280.0], phases=[100, 7, 0, 3, 1000],
         iters=[100, 100, 50, 100, 100]),
    dict(name="planar1000", graph=("planar_like", dict(n=1000, seed=4)), seeds=list(range(16)),
         t0s=[LADDER[i % 8] for i in range(16)], phases=FULL, iters=[400] * 8),
]


def weighted_graph():
    import rfmf_gb300 as R
    rng = np.random.default_rng(5)
    u = rng.integers(0, 300, 1500)
    v = rng.integers(0, 300, 1500)
    w = rng.integers(1, 6, 1500) * np.where(rng.random(1500) < 0.5, -1, 1)
    return R.csr_from_edges(u, v, w, name="weighted300")


def psha(s):
    return hashlib.sha256("".join("0" if x < 0 else "1" for x in s).encode()).hexdigest()


def build_graph(spec):
    import rfmf_gb300.graphs as G
    if spec == "weighted300":
        return weighted_graph()
    fn, kw = spec
    return getattr(G, fn)(**kw)


def main():
    import oracle as ora
    import refgpu
    import rfmf_gb300 as R
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    cases = CASES + [dict(name="weighted300", graph="weighted300", seeds=[1, 2, 3, 4],
                          t0s=[35.0, 70.0, 140.0, 280.0], phases=[64, 16, 4, 1],
                          iters=[200, 200, 200, 200])]
    out = []
    for c in cases:
        g = build_graph(c["graph"])
        init = np.stack([ora.initial_spins(s, g.n) for s in c["seeds"]])
        solver = [R.solver_seed(s) for s in c["seeds"]]
        r = refgpu.run(g, init, c["t0s"], solver, c["phases"], c["iters"], sms)
        o = ora.anneal(g, init, c["t0s"], solver, c["phases"], c["iters"])
        same = all(np.array_equal(r[k], o[k]) for k in ("end_spins", "best_spins", "cur_vals",
                                                         "best_vals"))
        h = hashlib.sha256(g.offsets.tobytes() + g.col.tobytes() + g.weight.tobytes()).hexdigest()
        rec = dict(c, n=g.n, m=g.m, csr_sha256=h, reference_kernel=dict(
            tpb=r["tpb"], choices={k: (bool(v) if isinstance(v, (bool, np.bool_)) else int(v))
                                   for k, v in r["choices"].items()},
            ms=round(r["ms"], 3)),
            best=[int(x) for x in r["best_vals"]], final=[int(x) for x in r["cur_vals"]],
            best_partition_sha256=[psha(x) for x in r["best_spins"]],
            final_partition_sha256=[psha(x) for x in r["end_spins"]],
            oracle_matches_reference_kernel=bool(same))
        print(c["name"], "oracle==reference kernel:", same, "tpb", r["tpb"], r["choices"], flush=True)
        out.append(rec)
    (HERE / "refkernel_runs.json").write_text(json.dumps(dict(cases=out), indent=0) + "\n")
    return 0 if all(x["oracle_matches_reference_kernel"] for x in out) else 1


if __name__ == "__main__":
    sys.exit(main())
