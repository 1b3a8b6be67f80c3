#!/usr/bin/env python3
"""Rerun chains of the reference's committed result logs on the GPU.

Test infrastructure.  Input: a spec written by
`oracle/pin_committed_logs.py RESULTS GRAPH all --spec SPEC.json` (run
parameters and expected cuts / partition hashes of every chain, read from the
reference's committed logs) and a directory holding the Gset graph files it
names.  Every chain of the spec runs through librfmf.so in one multi-graph
batch (advanced in windows of --window sweeps per launch); the best and final
cut values and the sha256 of both partition strings ("0"/"1" per vertex, the
log's format) are compared with the committed values and the outcome is
merged into tests/golden/committed_log_pin.json under "gpu_entries".

With --device-ingest the graphs are read by the native parser
(rfmf_gset_parse) and their CSR is built on the GPU (rfmf_graph_from_edges)
instead of by the Python reader, so the rerun also covers the ingest path.

Usage: pin_committed_logs_gpu.py SPEC.json GSET_DIR [--window N] [--device-ingest]
"""
import argparse
import hashlib
import json
import pathlib
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
OUT = HERE / "committed_log_pin.json"


def sha(s):
    return hashlib.sha256(s.encode()).hexdigest()


def partition(spins):
    return "".join("0" if s < 0 else "1" for s in spins)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("spec")
    ap.add_argument("gset_dir")
    ap.add_argument("--window", type=int, default=5_000_000)
    ap.add_argument("--device-ingest", action="store_true")
    a = ap.parse_args()

    import rfmf_gb300 as R

    spec = json.loads(pathlib.Path(a.spec).read_text())["chains"]
    sched = {(tuple(c["phases"]), tuple(c["iters"])) for c in spec}
    assert len(sched) == 1, "one schedule per batch"
    phases, iters = [list(x) for x in sched.pop()]
    total = sum(i for p, i in zip(phases, iters) if p)

    ctx = R.Context(0)
    graphs, dgs = {}, {}
    class Shape:   # n of a device-built graph (the host never holds its CSR)
        def __init__(self, n):
            self.n = n

    for c in spec:
        if c["graph"] not in graphs:
            path = pathlib.Path(a.gset_dir) / c["graph"]
            if a.device_ingest:
                d = R.parse_gset(path)
                dg = R.DeviceGraph.from_edges(ctx, d["u"], d["v"], d["w"])
                graphs[c["graph"]] = Shape(dg.n)
                dgs[c["graph"]] = dg
            else:
                g = R.read_gset(path, name=c["graph"])
                graphs[c["graph"]] = g
                dgs[c["graph"]] = R.DeviceGraph(ctx, g)
    init = [R.initial_spins(c["seed"], graphs[c["graph"]].n) for c in spec]
    b = R.Batch(ctx, [dgs[c["graph"]] for c in spec], [c["t0"] for c in spec],
                [R.solver_seed(c["seed"]) for c in spec], init, phases, iters)
    print(json.dumps(dict(chains=len(spec), total_sweeps=total, plan=b.info())), flush=True)

    t = time.time()
    done = 0
    while done < total:
        w = min(a.window, total - done)
        b.run(w)
        b.synchronize()
        done += w
        print(f"{done}/{total} sweeps, {time.time() - t:.1f} s", flush=True)
    el = time.time() - t
    r = b.read()

    entries = []
    for k, c in enumerate(spec):
        got = dict(best=int(r["best_vals"][k]), final=int(r["cur_vals"][k]),
                   best_partition_sha256=sha(partition(r["best_spins"][k])),
                   final_partition_sha256=sha(partition(r["end_spins"][k])))
        e = dict(results=c["results"], graph=c["graph"], chain=c["chain"], seed=c["seed"],
                 t0=c["t0"], n=graphs[c["graph"]].n, expected=c["expected"], gpu=got,
                 match=(got == c["expected"]))
        entries.append(e)
    nmatch = sum(e["match"] for e in entries)
    print(json.dumps(dict(matched=nmatch, of=len(entries), seconds=round(el, 1))), flush=True)

    record = json.loads(OUT.read_text()) if OUT.exists() else {"entries": []}
    keys = {(e["results"], e["graph"], e["chain"]) for e in entries}
    record["gpu_entries"] = [x for x in record.get("gpu_entries", [])
                             if (x["results"], x["graph"], x["chain"]) not in keys] + entries
    import torch
    runs = record.get("gpu_runs", {})
    if "gpu_run" in record:     # single-run records kept before per-set runs
        runs.setdefault("V100-SXM2-10M", record.pop("gpu_run"))
    for rs in sorted({c["results"] for c in spec}):
        runs[rs] = dict(device=torch.cuda.get_device_name(0), sm_count=ctx.info()["sm_count"],
                        chains=len(entries), sweeps_per_chain=total,
                        seconds=round(el, 1), window=a.window,
                        ingest="native parser + CSR built on the GPU" if a.device_ingest
                        else "Python reader + host CSR")
    record["gpu_runs"] = runs
    OUT.write_text(json.dumps(record, indent=1) + "\n")
    return 0 if nmatch == len(entries) else 1


if __name__ == "__main__":
    sys.exit(main())
