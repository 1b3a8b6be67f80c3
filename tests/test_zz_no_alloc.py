"""rfmf_anneal_noalloc: the annealer for callers that cannot allocate device
memory (their allocator owns all of it, or they must not allocate in the
middle of their own work).  It takes the caller's device buffers and keeps
its scratch in a fixed device array inside librfmf.so.

Checked through the C ABI against the allocating entry point rfmf_anneal on
the same inputs, at the suite's tolerance for this integer path (zero: every
spin and cut identical), on two calls in a row (the scratch array keeps the
previous call's contents), for each kernel variant the entry point picks:
int8 gains with compact int32 keys (+-1 weights), int32 gains (a weighted
graph whose max weighted degree is above 127) and the int64 score path (a
t0 small enough that the compact keys would overflow).  The entry point also
refuses, with a status and without a fault, a CSR whose check fails on the
device and a pointer off its alignment.  Collected last on purpose; it also
passes alone in a fresh process, where its first call performs the one-time
set-up."""
import numpy as np
import pytest

from conftest import chains_for

pytestmark = pytest.mark.gpu

RFMF_ERR_INVALID = 1
RFMF_ERR_CAPACITY = 4


def _bits(spins):
    """(C, n) +-1 int8 -> (C, ceil(n/32)) uint32 words, bit v = spin +1."""
    C, n = spins.shape
    words = (n + 31) // 32
    out = np.zeros((C, words), np.uint32)
    for v in range(n):
        out[:, v >> 5] |= (spins[:, v] > 0).astype(np.uint32) << np.uint32(v & 31)
    return out


def _unbits(words, n):
    v = np.arange(n)
    return np.where((words[:, v >> 5] >> (v & 31).astype(np.uint32)) & 1, 1, -1).astype(np.int8)


def _weighted_graph(rfmf, n, avg_degree, wmax, seed):
    """Erdos-Renyi graph with integer weights uniform in +-[1, wmax]."""
    rng = np.random.default_rng(seed)
    m = int(n * avg_degree / 2)
    u = rng.integers(0, n, m)
    v = rng.integers(0, n, m)
    keep = u != v
    u, v = u[keep], v[keep]
    w = rng.integers(1, wmax + 1, len(u)) * rng.choice([-1, 1], len(u))
    return rfmf.csr_from_edges(u, v, w, name=f"er{n}_w{wmax}")


class _Caller:
    """A caller that owns its device memory (here allocated with torch) and
    runs rfmf_anneal_noalloc over it."""

    def __init__(self, rfmf, g, t0s, phases, iters, solver):
        import torch
        self.torch = torch
        self.L = rfmf.lib()
        self.g = g
        dev = torch.device("cuda", 0)
        self.dev = dev
        self.off = torch.from_numpy(g.offsets.astype(np.int32)).to(dev)
        self.edges = torch.from_numpy(
            np.stack([g.col, g.weight], 1).astype(np.int32).ravel()).to(dev)
        total = sum(i for p, i in zip(phases, iters) if p)
        end, val, first = rfmf.beta_tables(t0s, total)
        starts = sorted(set(int(x) for x in first))
        runs_of = {s: (starts[i + 1] if i + 1 < len(starts) else len(end)) - s
                   for i, s in enumerate(starts)}
        self.chain_off = np.array([int(x) for x in first], np.int64)
        self.chain_runs = np.array([runs_of[int(x)] for x in first], np.int64)
        self.runs = len(end)
        self.d_end = torch.from_numpy(end).to(dev)
        self.d_val = torch.from_numpy(val).to(dev)
        self.sd = np.array(solver, np.uint64)
        self.t0a = np.array(t0s, np.float64)
        self.ph = np.array(phases, np.uint64)
        self.it = np.array(iters, np.uint64)

    def call(self, init, B, edges_ptr=None):
        torch = self.torch
        C = init.shape[0]
        spin_bits = torch.from_numpy(_bits(init).view(np.int32)).to(self.dev)
        best_bits = torch.zeros_like(spin_bits)
        cur = torch.zeros(C, dtype=torch.int64, device=self.dev)
        best = torch.zeros(C, dtype=torch.int64, device=self.dev)
        torch.cuda.synchronize()
        rc = self.L.rfmf_anneal_noalloc(
            0, None, self.g.n, self.off.data_ptr(),
            self.edges.data_ptr() if edges_ptr is None else edges_ptr, B, C,
            self.t0a.ctypes.data, self.sd.ctypes.data, len(self.ph), self.ph.ctypes.data,
            self.it.ctypes.data, self.d_end.data_ptr(), self.d_val.data_ptr(), self.runs,
            self.chain_off.ctypes.data, self.chain_runs.ctypes.data, spin_bits.data_ptr(),
            best_bits.data_ptr(), cur.data_ptr(), best.data_ptr())
        words = (self.g.n + 31) // 32
        out = dict(end=_unbits(spin_bits.cpu().numpy().view(np.uint32).reshape(C, words), self.g.n),
                   best=_unbits(best_bits.cpu().numpy().view(np.uint32).reshape(C, words), self.g.n),
                   cur=cur.cpu().numpy(), best_vals=best.cpu().numpy())
        return rc, out


CASES = {
    # +-1 weights, B <= 127: int8 gains, compact int32 keys
    "int8_gains": dict(graph=lambda R: R.erdos_renyi(700, 0.02, signed=True, seed=31),
                       t0s=[35.0, 50.0, 70.0, 100.0, 140.0, 200.0, 280.0, 400.0] * 8,
                       phases=[128, 32, 8, 3, 1], iters=[120] * 5),
    # weights up to +-40 on mean degree 12: B > 127, int32 gains
    "int32_gains": dict(graph=lambda R: _weighted_graph(R, 600, 12, 40, seed=7),
                        t0s=[2000.0, 4000.0, 8000.0, 16000.0] * 8,
                        phases=[64, 16, 4, 1], iters=[150] * 4),
    # t0 = 0.05: beta * B overflows the compact int32 key, int64 score path
    "int64_scores": dict(graph=lambda R: R.torus(20, 30, signed=True, seed=3),
                         t0s=[0.05, 0.07] * 16,
                         phases=[16, 4, 1], iters=[200] * 3),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_noalloc_matches_allocating_entry_point(rfmf, ctx, case):
    spec = CASES[case]
    g = spec["graph"](rfmf)
    t0s, phases, iters = spec["t0s"], spec["phases"], spec["iters"]
    C = len(t0s)
    seeds = list(range(100, 100 + C))
    init, solver = chains_for(g, seeds)
    B = g.max_weighted_degree()
    if case == "int32_gains":
        assert B > 127
    if case == "int64_scores":
        # (beta_max * B + max|gumbel|) * 2^kb >= 2^31 at kb = 4 (n = 600, one warp)
        import math
        bmax = round(math.log(1 + sum(iters)) / min(t0s) * 2**20)
        assert (bmax * B + 3617614) * 16 >= 2**31

    # the allocating path
    dg = rfmf.DeviceGraph(ctx, g)
    ref = rfmf.anneal_gpu(ctx, dg, B, init, t0s, phases, iters, solver)
    dg.close()

    caller = _Caller(rfmf, g, t0s, phases, iters, solver)
    for call in range(2):
        rc, got = caller.call(init, B)
        assert rc == 0, caller.L.rfmf_last_error().decode()
        assert np.array_equal(got["end"], ref.end_spins), (case, call)
        assert np.array_equal(got["best"], ref.best_spins), (case, call)
        assert np.array_equal(got["cur"], ref.final_vals), (case, call)
        assert np.array_equal(got["best_vals"], ref.best_vals), (case, call)


def test_noalloc_rejects_bad_csr_and_understated_bound(rfmf, ctx):
    """The on-device check refuses a CSR with a neighbour id out of range and
    a max_weighted_deg below the graph's own; a good call afterwards still
    equals the allocating path (the refused calls left nothing behind)."""
    import torch
    g = rfmf.erdos_renyi(300, 0.03, signed=True, seed=5)
    t0s = [35.0, 70.0, 140.0, 280.0]
    phases, iters = [8, 1], [100, 100]
    init, solver = chains_for(g, [1, 2, 3, 4])
    B = g.max_weighted_degree()
    caller = _Caller(rfmf, g, t0s, phases, iters, solver)

    rc, _ = caller.call(init, B - 1)
    assert rc == RFMF_ERR_INVALID, rc
    assert b"max_weighted_deg" in caller.L.rfmf_last_error()

    bad = caller.edges.clone()
    bad[2 * 5] = g.n + 7          # entry 5's neighbour id, out of range
    rc, _ = caller.call(init, B, edges_ptr=bad.data_ptr())
    assert rc == RFMF_ERR_INVALID, rc
    torch.cuda.synchronize()

    rc, got = caller.call(init, B)
    assert rc == 0, caller.L.rfmf_last_error().decode()
    dg = rfmf.DeviceGraph(ctx, g)
    ref = rfmf.anneal_gpu(ctx, dg, B, init, t0s, phases, iters, solver)
    dg.close()
    assert np.array_equal(got["best"], ref.best_spins)
    assert np.array_equal(got["best_vals"], ref.best_vals)


def test_noalloc_rejects_misaligned_pointer(rfmf):
    """A CSR entry pointer off its 8-byte boundary is refused on the host,
    before any device work."""
    g = rfmf.erdos_renyi(64, 0.1, signed=True, seed=2)
    init, solver = chains_for(g, [1])
    caller = _Caller(rfmf, g, [50.0], [2, 1], [10, 10], solver)
    rc, _ = caller.call(init, g.max_weighted_degree(), edges_ptr=caller.edges.data_ptr() + 4)
    assert rc == RFMF_ERR_INVALID
    assert b"misaligned" in caller.L.rfmf_last_error()


def test_noalloc_rejects_oversize(rfmf):
    L = rfmf.lib()
    one = np.zeros(8, np.int64)
    p = one.ctypes.data
    rc = L.rfmf_anneal_noalloc(0, None, 10, p, p, 1, 5000, p, p, 1, p, p, p, p, 1, p, p, p, p,
                               p, p)
    assert rc == RFMF_ERR_CAPACITY and b"4096" in L.rfmf_last_error()
