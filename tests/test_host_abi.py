"""librfmf.so on a machine without a GPU: it loads, exports every symbol
include/*.h declares, and its host-side helpers (the restated
src/host_common.cpp / src/max_cut.cpp / src/rng.hpp functions) match the
reference's fixtures.  No kernel is launched here."""
import ctypes as ct
import hashlib
import json
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def header_functions():
    """Every rfmf_* function the C headers (include/*.h) declare."""
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(rfmf_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_exports_every_declared_symbol(rfmf):
    L = rfmf.lib()
    names = header_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(L, name), name
    from rfmf_gb300._lib import SIGNATURES
    assert sorted(n for n, _, _ in SIGNATURES) == names


def test_version(rfmf):
    assert "sm_103a" in rfmf.version()


def test_no_device_reports_error(rfmf):
    """Context creation without a GPU fails with a status, not a crash."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(rfmf.RfmfError):
        rfmf.Context(0)


def test_beta_tables_match_reference(rfmf):
    for e in json.loads((GOLDEN / "beta_tables.json").read_text())["tables"]:
        end, val, off = rfmf.beta_tables(e["t0s"], e["total"])
        assert len(end) == e["runs"], e["t0s"]
        h = hashlib.sha256(end.tobytes() + val.tobytes()).hexdigest()
        assert h == e["sha256"], (e["t0s"], e["total"])
        assert [int(x) for x in off] == e["chain_off"]


def test_beta_tables_equal_per_step_schedule(rfmf, oracle):
    end, val, off = rfmf.beta_tables([35.0, 0.5, 400.0], 5000)
    bounds = list(off) + [len(end)]
    for c, t0 in enumerate([35.0, 0.5, 400.0]):
        E, V = end[bounds[c]:bounds[c + 1]], val[bounds[c]:bounds[c + 1]]
        idx = np.searchsorted(E, np.arange(5000), side="right")
        assert np.array_equal(V[idx], [oracle.beta_fixed(s + 1, t0) for s in range(5000)])


def test_beta_run_cap(rfmf):
    with pytest.raises(rfmf.RfmfError) as ei:
        rfmf.beta_tables([0.02], 10**8)
    assert ei.value.code == 6


def test_beta_overflow_refused(rfmf):
    """beta_fixed past int32 is undefined in the reference; refused here."""
    with pytest.raises(rfmf.RfmfError) as ei:
        rfmf.beta_tables([1e-3], 50)
    assert ei.value.code == 1


def test_score_gate(rfmf):
    for T, t0, B, ok in json.loads((GOLDEN / "score_gate.json").read_text())["cases"]:
        assert rfmf.score_safe_int32(T, t0, B) == bool(ok)


def test_initial_spins(rfmf):
    for e in json.loads((GOLDEN / "initial_spins.json").read_text())["cases"]:
        s = rfmf.initial_spins(e["seed"], e["n"])
        assert "".join("1" if x > 0 else "0" for x in s) == e["bits"]


def test_total_steps(rfmf):
    assert rfmf.total_steps([1, 2, 3]) == 6
    with pytest.raises(rfmf.RfmfError):
        rfmf.total_steps([10**12, 1])


def test_cut_and_degree(rfmf, oracle):
    g = rfmf.erdos_renyi(300, 0.05, signed=True, seed=3)
    for seed in range(5):
        s = oracle.initial_spins(seed, g.n)
        assert rfmf.cut_value(g, s) == oracle.cut_value(g, s) == g.cut_value(s)
    assert rfmf.max_weighted_degree(g) == oracle.max_weighted_degree(g) == g.max_weighted_degree()


def validate(rfmf, n, off, col, w):
    B = ct.c_int64(-1)
    off = np.asarray(off, np.uint32)
    col = np.asarray(col, np.int32)
    w = np.asarray(w, np.int32)
    rc = rfmf.lib().rfmf_csr_validate(n, off.ctypes.data, col.ctypes.data, w.ctypes.data,
                                      ct.byref(B))
    return rc, B.value


def test_csr_validation(rfmf):
    g = rfmf.erdos_renyi(100, 0.1, signed=True, seed=2)
    assert validate(rfmf, g.n, g.offsets, g.col, g.weight) == (0, g.max_weighted_degree())
    assert validate(rfmf, 2, [0, 1, 1], [1], [1])[0] == 1            # asymmetric
    assert validate(rfmf, 2, [0, 1, 2], [1, 0], [1, 2])[0] == 1      # unequal weights
    assert validate(rfmf, 2, [0, 1, 2], [0, 1], [1, 1])[0] == 1      # self loops
    assert validate(rfmf, 3, [0, 2, 3, 4], [2, 1, 0, 0], [1, 1, 1, 1])[0] == 1  # unsorted row
    assert validate(rfmf, 2, [0, 1, 2], [5, 0], [1, 1])[0] == 1      # id out of range
    assert validate(rfmf, 2, [0, 1, 2], [1, 0], [0, 0])[0] == 1      # zero weight
    assert validate(rfmf, 2, [1, 1, 2], [1, 0], [1, 1])[0] == 1      # offsets[0] != 0
    assert validate(rfmf, 0, [0], [], [])[0] == 0                    # empty graph
    assert validate(rfmf, 2, [0, 2, 4], [1, 1, 0, 0], [1, 1, 1, 1])[0] == 1   # duplicate entry
    assert validate(rfmf, 3, [0, 2, 1, 4], [1, 2, 0, 0], [1, 1, 1, 1])[0] == 1  # offsets decrease
    assert validate(rfmf, 2, [0, 1, 2], [1, 0], [2**31 - 1] * 2) == (0, 2**31 - 1)  # int32 max
    assert validate(rfmf, 2, [0, 1, 2], [1, 0], [-2**31] * 2)[0] == 4  # |w| beyond int32
    L = rfmf.lib()
    h = ct.c_void_p()
    assert L.rfmf_graph_create(None, 2, None, None, None, ct.byref(h)) == 1
