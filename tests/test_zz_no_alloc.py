"""rfmf_anneal_noalloc: the annealer for callers that cannot allocate device
memory (their allocator owns all of it, or they must not allocate in the
middle of their own work).  It takes the caller's device buffers and keeps
its scratch in a fixed device array inside librfmf.so.

Checked through the C ABI against the allocating entry point rfmf_anneal on
the same inputs, at the suite's tolerance for this integer path (zero: every
spin and cut identical), on two calls in a row (the scratch array keeps the
previous call's contents).  Collected last on purpose; it also passes alone
in a fresh process, where its first call performs the one-time set-up."""
import numpy as np
import pytest

from conftest import chains_for

pytestmark = pytest.mark.gpu


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


def test_noalloc_matches_allocating_entry_point(rfmf, ctx):
    import torch

    L = rfmf.lib()
    g = rfmf.erdos_renyi(700, 0.02, signed=True, seed=31)
    seeds = list(range(100, 164))
    t0s = [35.0, 50.0, 70.0, 100.0, 140.0, 200.0, 280.0, 400.0] * 8
    phases, iters = [128, 32, 8, 3, 1], [120, 120, 120, 120, 120]
    init, solver = chains_for(g, seeds)
    B = g.max_weighted_degree()

    # the allocating path
    dg = rfmf.DeviceGraph(ctx, g)
    ref = rfmf.anneal_gpu(ctx, dg, B, init, t0s, phases, iters, solver)

    # caller-owned device buffers (allocated by the caller, here with torch)
    dev = torch.device("cuda", 0)
    off = torch.from_numpy(g.offsets.astype(np.int32)).to(dev)
    edges = torch.from_numpy(np.stack([g.col, g.weight], 1).astype(np.int32).ravel()).to(dev)
    total = sum(i for p, i in zip(phases, iters) if p)
    end, val, first = rfmf.beta_tables(t0s, total)
    starts = sorted(set(int(x) for x in first))
    runs_of = {s: (starts[i + 1] if i + 1 < len(starts) else len(end)) - s
               for i, s in enumerate(starts)}
    chain_off = np.array([int(x) for x in first], np.int64)
    chain_runs = np.array([runs_of[int(x)] for x in first], np.int64)
    d_end = torch.from_numpy(end).to(dev)
    d_val = torch.from_numpy(val).to(dev)
    sd = np.array(solver, np.uint64)
    t0a = np.array(t0s, np.float64)
    ph = np.array(phases, np.uint64)
    it = np.array(iters, np.uint64)
    C = len(seeds)
    words = (g.n + 31) // 32

    for call in range(2):
        spin_bits = torch.from_numpy(_bits(init).view(np.int32)).to(dev)
        best_bits = torch.zeros_like(spin_bits)
        cur = torch.zeros(C, dtype=torch.int64, device=dev)
        best = torch.zeros(C, dtype=torch.int64, device=dev)
        torch.cuda.synchronize()
        rc = L.rfmf_anneal_noalloc(
            0, None, g.n, off.data_ptr(), edges.data_ptr(), B, C, t0a.ctypes.data,
            sd.ctypes.data, len(ph), ph.ctypes.data, it.ctypes.data, d_end.data_ptr(),
            d_val.data_ptr(), chain_off.ctypes.data, chain_runs.ctypes.data,
            spin_bits.data_ptr(), best_bits.data_ptr(), cur.data_ptr(), best.data_ptr())
        assert rc == 0, L.rfmf_last_error().decode()
        got_end = _unbits(spin_bits.cpu().numpy().view(np.uint32).reshape(C, words), g.n)
        got_best = _unbits(best_bits.cpu().numpy().view(np.uint32).reshape(C, words), g.n)
        assert np.array_equal(got_end, ref.end_spins), call
        assert np.array_equal(got_best, ref.best_spins), call
        assert np.array_equal(cur.cpu().numpy(), ref.final_vals), call
        assert np.array_equal(best.cpu().numpy(), ref.best_vals), call


def test_noalloc_rejects_oversize(rfmf):
    L = rfmf.lib()
    one = np.zeros(8, np.int64)
    rc = L.rfmf_anneal_noalloc(0, None, 10, one.ctypes.data, one.ctypes.data, 1, 5000,
                               one.ctypes.data, one.ctypes.data, 1, one.ctypes.data,
                               one.ctypes.data, one.ctypes.data, one.ctypes.data,
                               one.ctypes.data, one.ctypes.data, one.ctypes.data,
                               one.ctypes.data, one.ctypes.data, one.ctypes.data)
    assert rc == 4 and b"4096" in L.rfmf_last_error()
