"""Graph ingest on the host side: the native Gset/MQLib parser
(rfmf_gset_parse) plus the CSR builder reproduce the reference's loader
(src/read_gset.cpp + src/graph.cpp + src/immutable_graph.hpp) on the
synthetic cases of tests/golden/ingest_cases.json, whose expected CSR digests
were produced by the reference's own code (tests/golden/make_ingest_golden.py)."""
import hashlib
import json
import pathlib

import numpy as np
import pytest

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
CASES = json.loads((GOLDEN / "ingest_cases.json").read_text())["cases"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_parser_and_csr_match_reference_loader(rfmf, case):
    d = rfmf.parse_gset(case["text"])
    assert d["scale"] == case["scale"]
    assert d["zero_dropped"] == case["zero_dropped"]
    g = rfmf.csr_from_edges(d["u"], d["v"], d["w"])
    h = hashlib.sha256(g.offsets.astype(np.uint32).tobytes() + g.col.astype(np.int32).tobytes() +
                       g.weight.astype(np.int32).tobytes()).hexdigest()
    assert (g.n, g.m, g.max_weighted_degree(), h) == (case["n"], case["m"], case["B"], case["sha256"])


def test_parser_errors(rfmf):
    for bad in ["", "# only a comment\n", "3\n", "2 1\n1\n", "2 2\n1 2 1\n"]:
        with pytest.raises(rfmf.RfmfError):
            rfmf.parse_gset(bad)


def test_parser_forced_scale(rfmf):
    d = rfmf.parse_gset("2 1\n1 2 0.26\n", forced_scale=10.0)
    assert d["scale"] == 10.0 and list(d["w"]) == [3]


def _random_gset(rng, n, m, mode):
    lines = []
    for _ in range(m):
        a = rng.randint(0, n + (0 if rng.random() < 0.9 else 10**6))
        b = rng.randint(1, n)
        if a == b:
            b = a + 1
        if mode == "int":
            w = str(rng.choice([1, -1, 2, 0, 5, -7]))
        elif mode == "float":
            w = repr(round(rng.uniform(-10, 10), rng.randint(0, 6)))
        elif mode == "tiny":
            w = repr(rng.uniform(-1e-6, 1e-6))
        elif mode == "huge":
            w = str(rng.randint(-10**9, 10**9))
        elif mode == "hugefloat":
            w = repr(rng.uniform(-1e14, 1e14))
        else:
            w = rng.choice(["1", "-2", "0.5", "3.25", "1e-3", "0", "  7 ", "-0.0004"])
        lines.append(f"{a} {b} {w}")
    return f"# random\n{n} {m}\n" + "\n".join(lines) + "\n"


def test_parser_matches_reference_loader_random(rfmf, ref_host, tmp_path):
    """Random Gset texts (integral, fractional, tiny and huge weights; ids in
    and far out of the header's range) through the native parser + CSR
    builder and through the reference's own loader (oracle/_ref, built from
    its sources): same scale, same dropped-zero count, same CSR.  Texts the
    reference refuses must be refused too."""
    import ctypes as ct
    import random
    L = ref_host
    L.ref_gset_scale.restype = ct.c_double
    L.ref_gset_scale.argtypes = [ct.c_void_p]
    L.ref_gset_zero_dropped.restype = ct.c_int64
    L.ref_gset_zero_dropped.argtypes = [ct.c_void_p]
    rng = random.Random(2024)
    for case in range(120):
        mode = ["int", "float", "tiny", "huge", "hugefloat", "mixed"][case % 6]
        n = rng.choice([5, 50, 400, 2000])
        text = _random_gset(rng, n, rng.randint(1, 3 * n), mode)
        path = tmp_path / f"c{case}.txt"
        path.write_text(text)
        h = L.ref_gset_load(str(path).encode())
        try:
            d = rfmf.parse_gset(text)
        except rfmf.RfmfError:
            assert not h, (case, mode)
            continue
        assert h, (case, mode)
        assert d["scale"] == L.ref_gset_scale(h), (case, mode)
        assert d["zero_dropped"] == L.ref_gset_zero_dropped(h), (case, mode)
        rn, rm = L.ref_gset_n(h), L.ref_gset_m(h)
        off = np.zeros(rn + 1, np.uint32)
        col = np.zeros(2 * rm, np.int32)
        w = np.zeros(2 * rm, np.int32)
        L.ref_gset_copy(h, off.ctypes.data, col.ctypes.data, w.ctypes.data)
        L.ref_gset_free(h)
        g = rfmf.csr_from_edges(d["u"], d["v"], d["w"])
        assert g.n == rn and np.array_equal(g.offsets, off), (case, mode)
        assert np.array_equal(g.col, col) and np.array_equal(g.weight, w), (case, mode)


def test_injected_host_allocation_failure(rfmf):
    """The testing aid rfmf_debug_fail_host_alloc makes the countdown-th host
    allocation checkpoint fail; the call reports RFMF_ERR_NOMEM instead of
    ending the process, and the next call works (host only: the parser)."""
    text = "3 2\n1 2 1\n2 3 -1\n"
    rfmf.debug_fail_host_alloc(2)
    assert len(rfmf.parse_gset(text)["u"]) == 2          # first checkpoint passes
    with pytest.raises(rfmf.RfmfError) as ei:
        rfmf.parse_gset(text)                              # second one fails
    assert ei.value.code == 3
    assert len(rfmf.parse_gset(text)["u"]) == 2          # disarmed after firing
    rfmf.debug_fail_host_alloc(0)
