"""The oracle (CPU restatement) pinned against the reference's own host code.

Fixtures in tests/golden/ were produced by tests/golden/make_golden.py from
the reference's sources (oracle/_ref); where oracle/_ref is present the same
checks also run live against it.
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
