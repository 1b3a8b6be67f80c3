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
