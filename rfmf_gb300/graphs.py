"""Host-side graph input path: Gset/MQLib reader, CSR canonicalisation and
seeded synthetic generators of the shapes the reference benchmarks on.

The CSR follows the reference's load path exactly (src/host_common.cpp:
333-348 -> src/read_gset.cpp:98-241 -> src/graph.cpp:11-17 ->
src/immutable_graph.hpp:44-176): duplicate edges keep their FIRST weight,
degree-0 vertices are removed, surviving vertices are renumbered densely in
ascending original id, and every row is sorted ascending by neighbour.
"""
import math
from dataclasses import dataclass

import numpy as np


@dataclass
class CsrGraph:
    n: int
    offsets: np.ndarray   # uint32 [n+1]
    col: np.ndarray       # int32 [2m]
    weight: np.ndarray    # int32 [2m]
    name: str = ""
    orig_ids: np.ndarray = None   # dense id -> original id

    @property
    def m(self):
        return int(self.offsets[-1]) // 2

    def max_weighted_degree(self):
        if self.n == 0:
            return 0
        a = np.abs(self.weight.astype(np.int64))
        s = np.add.reduceat(a, self.offsets[:-1].astype(np.int64)) if len(a) else np.zeros(self.n, np.int64)
        deg = np.diff(self.offsets.astype(np.int64))
        s = np.where(deg > 0, s, 0)
        return int(s.max()) if len(s) else 0

    def cut_value(self, spin):
        spin = np.asarray(spin)
        src = np.repeat(np.arange(self.n), np.diff(self.offsets.astype(np.int64)))
        mask = (self.col > src) & (spin[src] != spin[self.col])
        return int(self.weight[mask].astype(np.int64).sum())


def csr_from_edges(u, v, w, name=""):
    """Canonical CSR from an undirected edge list (original vertex ids).

    First occurrence of a repeated edge wins (Graph::addEdge,
    src/graph.cpp:11-17); self loops are dropped; only vertices that carry an
    edge survive, renumbered by ascending original id."""
    u = np.asarray(u, np.int64)
    v = np.asarray(v, np.int64)
    w = np.asarray(w, np.int64)
    keep = u != v
    u, v, w = u[keep], v[keep], w[keep]
    a = np.minimum(u, v)
    b = np.maximum(u, v)
    if len(a):
        # stable unique on (a, b): first occurrence keeps its weight
        key = np.stack([a, b], 1)
        _, first = np.unique(key, axis=0, return_index=True)
        first = np.sort(first)
        a, b, w = a[first], b[first], w[first]
    ids = np.unique(np.concatenate([a, b])) if len(a) else np.zeros(0, np.int64)
    n = len(ids)
    ia = np.searchsorted(ids, a)
    ib = np.searchsorted(ids, b)
    src = np.concatenate([ia, ib])
    dst = np.concatenate([ib, ia])
    ww = np.concatenate([w, w])
    order = np.lexsort((dst, src))
    src, dst, ww = src[order], dst[order], ww[order]
    if len(ww) and (ww.max() > 2**31 - 1 or ww.min() < -2**31):
        raise ValueError("edge weight does not fit int32")
    offsets = np.zeros(n + 1, np.int64)
    np.add.at(offsets, src + 1, 1)
    offsets = np.cumsum(offsets)
    if offsets[-1] >= 2**32:
        raise ValueError("too many edges for uint32 offsets")
    return CsrGraph(n=n, offsets=offsets.astype(np.uint32), col=dst.astype(np.int32),
                    weight=ww.astype(np.int32), name=name, orig_ids=ids)


def read_gset(path, name=None):
    """Gset/MQLib text: '#'/blank lines skipped, header 'N M', then 'u v w'.

    Integral weights only (the reader's scale-1 path, src/read_gset.cpp:
    172-201); a non-integral weight raises (the reference rescales those by a
    power of ten, which this reader does not implement)."""
    lines = []
    with open(path) as f:
        for line in f:
            s = line.strip()
            if not s or s.startswith("#"):
                continue
            lines.append(s)
    if not lines:
        raise ValueError("no header line")
    hdr = lines[0].split()
    nhdr, mhdr = int(hdr[0]), int(hdr[1])
    if len(lines) - 1 < mhdr:
        raise ValueError(f"expected {mhdr} edges, found {len(lines) - 1}")
    arr = np.array([l.split()[:3] for l in lines[1:1 + mhdr]], dtype=object)
    u = arr[:, 0].astype(np.int64)
    v = arr[:, 1].astype(np.int64)
    wf = arr[:, 2].astype(np.float64)
    if np.any(np.floor(wf) != wf):
        raise ValueError("non-integral weights are not supported by this reader")
    w = wf.astype(np.int64)
    keep = w != 0
    g = csr_from_edges(u[keep], v[keep], w[keep], name=name or str(path).rsplit("/", 1)[-1])
    g.header_n = nhdr
    return g


# ---------------------------------------------------------------- synthetic
def _weights(rng, k, signed):
    if signed:
        return np.where(rng.random(k) < 0.5, -1, 1).astype(np.int64)
    return np.ones(k, np.int64)


def erdos_renyi(n, p, signed=False, seed=0, name=None):
    """G(n, p): every unordered pair an edge with probability p (the shape of
    Gset G1-G5 at n=800, p=0.06)."""
    rng = np.random.default_rng(seed)
    us, vs = [], []
    for i in range(n - 1):
        j = np.nonzero(rng.random(n - 1 - i) < p)[0] + i + 1
        us.append(np.full(len(j), i))
        vs.append(j)
    u = np.concatenate(us) if us else np.zeros(0, np.int64)
    v = np.concatenate(vs) if vs else np.zeros(0, np.int64)
    return csr_from_edges(u, v, _weights(rng, len(u), signed),
                          name=name or f"er{n}_p{p}")


def erdos_renyi_degree(n, avg_degree, signed=False, seed=0, name=None):
    return erdos_renyi(n, avg_degree / (n - 1), signed=signed, seed=seed,
                       name=name or f"er{n}_d{avg_degree}")


def torus(rows, cols, signed=False, seed=0, name=None):
    """2-D toroidal grid rows x cols: 2*rows*cols edges, degree 4 (the shape of
    Gset G48-G50, G62, G65-G67, G72, G77, G81)."""
    rng = np.random.default_rng(seed)
    idx = np.arange(rows * cols).reshape(rows, cols)
    right = np.roll(idx, -1, axis=1)
    down = np.roll(idx, -1, axis=0)
    u = np.concatenate([idx.ravel(), idx.ravel()])
    v = np.concatenate([right.ravel(), down.ravel()])
    return csr_from_edges(u, v, _weights(rng, len(u), signed),
                          name=name or f"torus{rows}x{cols}")


def random_tree(n, signed=False, seed=0, name=None):
    """Random recursive tree: vertex i > 0 attaches to a uniform earlier vertex;
    n-1 edges (the sparse, spanning-tree-like shape of Gset G70)."""
    rng = np.random.default_rng(seed)
    v = np.arange(1, n)
    u = (rng.random(n - 1) * v).astype(np.int64)
    return csr_from_edges(u, v, _weights(rng, n - 1, signed), name=name or f"tree{n}")


def planar_like(n, avg_degree=11.7, signed=False, seed=0, name=None):
    """Random geometric graph in the unit square with the connection radius
    set for the requested mean degree: spatially local like Gset's planar
    family G14-G17, G35-G38, G51-G54 (mean degree ~11.7).  Edges are every
    pair within the radius (k-d tree), weights drawn in sorted pair order."""
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    r = math.sqrt(avg_degree / (math.pi * (n - 1)))
    pairs = cKDTree(pts).query_pairs(r, output_type="ndarray")
    if len(pairs):
        pairs = pairs[np.lexsort((pairs[:, 1], pairs[:, 0]))]
    u = pairs[:, 0].astype(np.int64) if len(pairs) else np.zeros(0, np.int64)
    v = pairs[:, 1].astype(np.int64) if len(pairs) else np.zeros(0, np.int64)
    return csr_from_edges(u, v, _weights(rng, len(u), signed),
                          name=name or f"planar{n}")


def erdos_renyi_sparse(n, avg_degree, signed=False, seed=0, name=None):
    """G(n, p) with p = avg_degree / (n - 1) in O(n + m) time: geometric gaps
    between successive edges over the row-major upper-triangle pair index
    (Batagelj and Brandes 2005), for large sparse instances."""
    rng = np.random.default_rng(seed)
    p = avg_degree / (n - 1)
    N = n * (n - 1) // 2
    ks = []
    pos = -1
    while True:
        need = max(1024, int((N - pos) * p * 1.1) + 64)
        gaps = rng.geometric(p, size=need)
        idx = pos + np.cumsum(gaps)
        ks.append(idx[idx < N])
        if idx[-1] >= N:
            break
        pos = int(idx[-1])
    k = np.concatenate(ks).astype(np.int64)
    # row i starts at i*n - i*(i+1)/2 - i ... pair index of (i, j>i)
    starts = np.arange(n, dtype=np.int64)
    starts = starts * (2 * n - starts - 1) // 2
    u = np.searchsorted(starts, k, side="right") - 1
    v = k - starts[u] + u + 1
    return csr_from_edges(u, v, _weights(rng, len(u), signed),
                          name=name or f"er{n}_d{avg_degree}")
