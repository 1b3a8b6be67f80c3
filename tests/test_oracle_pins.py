"""The oracle (CPU restatement) pinned against the reference's own host code
and against recorded runs of the reference's own GPU kernel.

Fixtures in tests/golden/ were produced by tests/golden/make_golden.py from
the reference's sources (oracle/_ref); where oracle/_ref is present the same
checks also run live against it.  tests/golden/refkernel_runs.json holds runs
of the reference's mcKernel on a GB300, which the oracle reproduces here.
"""
import json

import numpy as np
import pytest

from conftest import GOLDEN


def load(name):
    return json.loads((GOLDEN / name).read_text())


def test_philox_kat(oracle):
    d = load("philox_kat.json")
    for e in d["blocks"]:
        out = oracle.philox_block(e["seed"], e["step"], e["block"])
        assert [int(x) for x in out] == e["out"], e


def test_gumbel_table(oracle):
    d = load("philox_kat.json")
    assert [oracle.gumbel(r) for r in range(2048)] == d["gumbel_by_field"]


def test_beta_fixed_samples(oracle):
    for e in load("beta_tables.json")["samples"]:
        assert oracle.beta_fixed(e["step"], e["t0"]) == e["beta"], e


def test_score_gate(oracle):
    for T, t0, B, ok in load("score_gate.json")["cases"]:
        assert oracle.score_safe_int32(T, t0, B) == bool(ok), (T, t0, B)


def test_initial_spins(oracle):
    for e in load("initial_spins.json")["cases"]:
        s = oracle.initial_spins(e["seed"], e["n"])
        assert "".join("1" if x > 0 else "0" for x in s) == e["bits"], e


def test_live_reference_primitives(oracle, ref_host):
    rng = np.random.default_rng(7)
    for _ in range(2000):
        seed = int(rng.integers(0, 2**63)) * 2 + int(rng.integers(0, 2))
        step = int(rng.integers(1, 2**40))
        block = int(rng.integers(0, 2**20))
        out = np.zeros(4, np.uint32)
        ref_host.ref_philox_block(seed, step, block, out.ctypes.data)
        assert np.array_equal(out, oracle.philox_block(seed, step, block))
    for s in [1, 7, 1000, 123456789]:
        for t0 in [0.5, 35.0, 77.7]:
            assert ref_host.ref_beta_fixed(s, t0) == oracle.beta_fixed(s, t0)


def test_committed_log_pin_record():
    """Record of oracle/pin_committed_logs.py: chains of the reference's
    committed V100 logs (8e7 sweeps each) rerun by the oracle; every recorded
    chain must have reproduced the committed cuts and partitions exactly."""
    p = GOLDEN / "committed_log_pin.json"
    if not p.exists():
        pytest.skip("no committed-log pin recorded yet")
    rec = json.loads(p.read_text())
    assert rec["entries"], "empty pin record"
    for e in rec["entries"]:
        assert e["match"], e
        assert e["expected"]["best"] == e["oracle"]["best"]
        assert e["expected"]["best_partition_sha256"] == e["oracle"]["best_partition_sha256"]


def test_committed_log_gpu_pin_record():
    """Record of tests/golden/pin_committed_logs_gpu.py: whole result logs of
    the reference (every chain of a graph, 8e7 sweeps each) rerun through
    librfmf.so on a GB300; each chain's cuts and partitions must equal the
    committed ones."""
    p = GOLDEN / "committed_log_pin.json"
    rec = json.loads(p.read_text()) if p.exists() else {}
    if not rec.get("gpu_entries"):
        pytest.skip("no GPU rerun of the committed logs recorded yet")
    for e in rec["gpu_entries"]:
        assert e["match"], e
        assert e["gpu"] == e["expected"]


def _refkernel_cases():
    import json
    p = GOLDEN / "refkernel_runs.json"
    cases = json.loads(p.read_text())["cases"] if p.exists() else []
    # every recorded case (chains x sweeps x n up to 2e9: seconds on a few cores)
    return [c for c in cases
            if len(c["seeds"]) * sum(i for P, i in zip(c["phases"], c["iters"]) if P) * c["n"] <= 2e9]


@pytest.mark.parametrize("case", _refkernel_cases(), ids=lambda c: c["name"])
def test_oracle_reproduces_reference_kernel_runs(oracle, case):
    """The oracle against the reference's own GPU kernel: runs of mcKernel
    (its sources built for sm_103a, launched with the reference host code's
    choices on a GB300; tests/golden/make_refkernel_golden.py) recorded best
    and final cuts and partition digests, which the oracle must reproduce
    exactly on the same graph, seeds and schedule."""
    import hashlib
    import sys

    from conftest import ROOT, chains_for
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    import make_refkernel_golden as M

    g = M.build_graph(case["graph"] if case["graph"] == "weighted300" else tuple(case["graph"]))
    assert hashlib.sha256(g.offsets.tobytes() + g.col.tobytes() +
                          g.weight.tobytes()).hexdigest() == case["csr_sha256"]
    init, solver = chains_for(g, case["seeds"])
    r = oracle.anneal(g, init, case["t0s"], solver, case["phases"], case["iters"])
    assert [int(x) for x in r["best_vals"]] == case["best"]
    assert [int(x) for x in r["cur_vals"]] == case["final"]
    assert [M.psha(x) for x in r["best_spins"]] == case["best_partition_sha256"]
    assert [M.psha(x) for x in r["end_spins"]] == case["final_partition_sha256"]
