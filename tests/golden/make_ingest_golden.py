#!/usr/bin/env python3
"""Golden vectors for graph ingest: synthetic Gset-format texts run through
the reference's own loader (src/read_gset.cpp read_instance_from_file ->
degree-0 removal -> AnnealCsr, via oracle/_ref/libref_host.so built by
oracle/build_ref.sh from the reference's sources).

Each case stores the text itself (synthetic, generated below from a seed)
and what the reference produced: n, m, B, scale, zero-dropped count and the
sha256 of offsets|col|weight.  tests/test_ingest.py checks the native parser
plus the host CSR builder against them on the CPU, and
tests/test_gpu_ingest.py the device CSR build.

Cases cover comment and blank lines, CRLF line ends, duplicate edges in both
directions with different weights (first wins), zero weights, gapped and
unordered ids, negative weights, fractional weights (power-of-ten scaling)
and weights that round to zero after scaling.
"""
import ctypes as ct
import hashlib
import json
import pathlib
import random
import sys
import tempfile

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
OUT = HERE / "ingest_cases.json"
P, I64 = ct.c_void_p, ct.c_int64


def cases():
    out = []
    out.append(("hand", "# comment\n\n5 7\n1 2 1\n2 3 -2\n# inside\n3 1 4\n2 1 7\r\n"
                        "4 5 0\n100000 5 3\n17 3 -1\n"))
    out.append(("float", "4 5\n1 2 0.5\n2 3 -1.25\n3 4 3.75\n4 1 0.001\n1 3 2\n"))
    out.append(("round_to_zero", "3 4\n1 2 1000.25\n2 3 0.0004\n1 3 -7.5\n3 1 9\n"))
    rng = random.Random(11)
    lines = []
    ids = rng.sample(range(1, 5000), 300)
    for _ in range(2000):
        a, b = rng.sample(ids, 2)
        w = rng.choice([1, -1, 1, 2, -3, 0])
        lines.append(f"{a} {b} {w}")
    out.append(("random_sparse_ids", f"5000 {len(lines)}\n" + "\n".join(lines) + "\n"))
    rng = random.Random(12)
    lines = []
    for _ in range(1500):
        a, b = rng.sample(range(0, 400), 2)
        w = round(rng.uniform(-5, 5), 3)
        lines.append(f"{a} {b} {w}")
    out.append(("random_float", f"400 {len(lines)}\n" + "\n".join(lines) + "\n"))
    return out


def main():
    L = ct.CDLL(str(ROOT / "oracle" / "_ref" / "libref_host.so"))
    L.ref_gset_load.restype = P
    L.ref_gset_load.argtypes = [ct.c_char_p]
    for f in ("ref_gset_n", "ref_gset_m", "ref_gset_zero_dropped"):
        getattr(L, f).restype = I64
        getattr(L, f).argtypes = [P]
    L.ref_gset_scale.restype = ct.c_double
    L.ref_gset_scale.argtypes = [P]
    L.ref_gset_copy.argtypes = [P, P, P, P]
    recs = []
    for name, text in cases():
        with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
            f.write(text)
            path = f.name
        h = L.ref_gset_load(path.encode())
        assert h, name
        n, m = L.ref_gset_n(h), L.ref_gset_m(h)
        off = np.zeros(n + 1, np.uint32)
        col = np.zeros(2 * m, np.int32)
        w = np.zeros(2 * m, np.int32)
        L.ref_gset_copy(h, off.ctypes.data, col.ctypes.data, w.ctypes.data)
        B = int(max((np.abs(w[off[v]:off[v + 1]].astype(np.int64)).sum() for v in range(n)),
                    default=0))
        recs.append(dict(name=name, text=text, n=int(n), m=int(m), B=B,
                         scale=L.ref_gset_scale(h), zero_dropped=int(L.ref_gset_zero_dropped(h)),
                         sha256=hashlib.sha256(off.tobytes() + col.tobytes() + w.tobytes()).hexdigest()))
        print(name, n, m, B, recs[-1]["scale"], recs[-1]["zero_dropped"])
    OUT.write_text(json.dumps({"cases": recs}, indent=1) + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
