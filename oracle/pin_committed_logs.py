#!/usr/bin/env python3
"""Pin the oracle's full sweep against the reference's committed result logs.

Test infrastructure, run in a checkout next to the reference (it reads the
reference's Gset graph files, results/*/reproduce.sh and results/*/logs/*.out).
For each selected chain it takes the seed, t0, phases and iters that produced
the committed V100 log line, reruns that chain through the oracle
(rfmf_oracle_anneal_window) for the full schedule, and compares the best and
final cut values and both partition strings byte for byte with the log.

The expected values (cuts and sha256 of the partition strings, never the
graphs) are written to tests/golden/committed_log_pin.json together with the
oracle's outcome, so the pin is on record without the reference present.

Usage: pin_committed_logs.py RESULTS_DIR GRAPH CHAIN[,CHAIN...]|all [--threads N]
  e.g. pin_committed_logs.py V100-SXM2-10M G62 0,1,2,3
With --spec OUT.json it runs nothing: it appends the selected chains' run
parameters and expected values (cuts, partition hashes) to OUT.json, the input
of tests/golden/pin_committed_logs_gpu.py, which reruns them on the GPU.
"""
import argparse
import ctypes as ct
import hashlib
import json
import os
import pathlib
import re
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REF = pathlib.Path(os.environ.get("RFMF_REFERENCE", "/root/reference"))
OUT = HERE.parent / "tests" / "golden" / "committed_log_pin.json"
SOLVER_SEED_OFFSET = 0xC2B2AE3D27D4EB4F  # src/host_common.h:25


def parse_reproduce(path, graph):
    for line in path.read_text().splitlines():
        if line.startswith("./main") and f"Gset/{graph} " in line:
            toks = line.split()
            arg = {toks[i]: toks[i + 1] for i in range(2, len(toks) - 1, 2)}
            return ([int(x) for x in arg["--seeds"].split(",")],
                    [float(x) for x in arg["--t0s"].split(",")],
                    [int(x) for x in arg["--phases"].split(",")],
                    [int(x) for x in arg["--iters"].split(",")])
    raise SystemExit(f"{graph} not in {path}")


def parse_log(path):
    chains = []
    lines = path.read_text().splitlines()
    for i, line in enumerate(lines):
        if line.startswith("device:"):
            m = re.search(r"--seed (\d+) .* --t0 ([0-9.]+) .*best-cut-value: (-?\d+) "
                          r"final-cut-value: (-?\d+)", line)
            best_p = lines[i + 1].split(": ", 1)[1]
            final_p = lines[i + 2].split(": ", 1)[1]
            chains.append(dict(seed=int(m.group(1)), t0=float(m.group(2)),
                               best=int(m.group(3)), final=int(m.group(4)),
                               best_partition=best_p, final_partition=final_p))
    return chains


def sha(s):
    return hashlib.sha256(s.encode()).hexdigest()


def expected_of(chain):
    return dict(best=chain["best"], final=chain["final"],
                best_partition_sha256=sha(chain["best_partition"]),
                final_partition_sha256=sha(chain["final_partition"]))


def write_spec(a):
    rdir = REF / "results" / a.results
    seeds, t0s, phases, iters = parse_reproduce(rdir / "reproduce.sh", a.graph)
    log = parse_log(rdir / "logs" / f"{a.graph}.out")
    sel = range(len(log)) if a.chains == "all" else [int(x) for x in a.chains.split(",")]
    out = pathlib.Path(a.spec)
    spec = json.loads(out.read_text()) if out.exists() else {"chains": []}
    for c in sel:
        assert log[c]["seed"] == seeds[c] and log[c]["t0"] == t0s[c]
        spec["chains"].append(dict(results=a.results, graph=a.graph, chain=c, seed=seeds[c],
                                   t0=t0s[c], phases=phases, iters=iters,
                                   expected=expected_of(log[c])))
    out.write_text(json.dumps(spec) + "\n")
    print(f"{len(sel)} chains of {a.results}/{a.graph} -> {out}")
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("results")
    ap.add_argument("graph")
    ap.add_argument("chains")
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--spec", default=None)
    a = ap.parse_args()
    if a.spec:
        return write_spec(a)

    sys.path.insert(0, str(HERE))
    import oracle as ora

    ref = ct.CDLL(str(HERE / "_ref" / "libref_host.so"))
    ref.ref_gset_load.restype = ct.c_void_p
    ref.ref_gset_load.argtypes = [ct.c_char_p]
    ref.ref_gset_n.restype = ct.c_int64
    ref.ref_gset_m.restype = ct.c_int64
    ref.ref_gset_n.argtypes = ref.ref_gset_m.argtypes = [ct.c_void_p]
    ref.ref_gset_copy.argtypes = [ct.c_void_p] * 4

    rdir = REF / "results" / a.results
    seeds, t0s, phases, iters = parse_reproduce(rdir / "reproduce.sh", a.graph)
    log = parse_log(rdir / "logs" / f"{a.graph}.out")
    h = ref.ref_gset_load(str(REF / "Gset" / a.graph).encode())
    n, m = ref.ref_gset_n(h), ref.ref_gset_m(h)

    class G:
        pass
    g = G()
    g.n = n
    g.offsets = np.zeros(n + 1, np.uint32)
    g.col = np.zeros(2 * m, np.int32)
    g.weight = np.zeros(2 * m, np.int32)
    ref.ref_gset_copy(h, g.offsets.ctypes.data, g.col.ctypes.data, g.weight.ctypes.data)

    sel = [int(x) for x in a.chains.split(",")]
    for c in sel:
        assert log[c]["seed"] == seeds[c] and log[c]["t0"] == t0s[c]
    init = np.stack([ora.initial_spins(seeds[c], n) for c in sel])
    t = time.time()
    res = ora.anneal(g, init, [t0s[c] for c in sel],
                     [(seeds[c] + SOLVER_SEED_OFFSET) % 2**64 for c in sel],
                     phases, iters, nthreads=a.threads)
    el = time.time() - t
    best, spins, bestv, cur = res["best_spins"], res["end_spins"], res["best_vals"], res["cur_vals"]

    record = json.loads(OUT.read_text()) if OUT.exists() else {"entries": []}
    record.setdefault("entries", [])
    for k, c in enumerate(sel):
        bp = "".join("0" if s < 0 else "1" for s in best[k])
        fp = "".join("0" if s < 0 else "1" for s in spins[k])
        e = dict(results=a.results, graph=a.graph, chain=c, seed=seeds[c], t0=t0s[c],
                 phases=phases, iters=iters, n=n, m=m,
                 expected=expected_of(log[c]),
                 oracle=dict(best=int(bestv[k]), final=int(cur[k]),
                             best_partition_sha256=sha(bp), final_partition_sha256=sha(fp),
                             seconds=round(el, 1)))
        e["match"] = (e["expected"] == {k2: v for k2, v in e["oracle"].items() if k2 != "seconds"})
        print(json.dumps(e))
        record["entries"] = [x for x in record["entries"]
                             if not (x["results"] == a.results and x["graph"] == a.graph
                                     and x["chain"] == c)] + [e]
    OUT.write_text(json.dumps(record, indent=1) + "\n")
    return 0 if all(x["match"] for x in record["entries"]) else 1


if __name__ == "__main__":
    sys.exit(main())
