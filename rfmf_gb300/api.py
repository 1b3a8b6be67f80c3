"""Python mirror of the reference's annealer interface over the C ABI.

Names and argument meanings follow the reference (gt-tinker/rfmf):
anneal_gpu <-> gpu3::annealGpu (src/anneal_gpu.cuh:76-88), LaunchConfig <->
gpu3::LaunchConfig (src/anneal_gpu.cuh:52-58), the helpers <->
src/host_common.h.  Every call goes through librfmf.so; errors raise
RfmfError instead of exiting.
"""
import ctypes as ct
from dataclasses import dataclass

import numpy as np

from ._lib import (REQUEST_STATES, BatchPlan, LaunchConfig, RequestStatus, RfmfError,
                   ServerConfig, ServerStats, check, lib)

# Offset between a chain's raw seed (initial spins) and its Philox solver seed
# (src/host_common.h:22-25, main.cu:27-29).
SOLVER_SEED_OFFSET = 0xC2B2AE3D27D4EB4F


def solver_seed(seed):
    return (int(seed) + SOLVER_SEED_OFFSET) % 2**64


def _p(a):
    return a.ctypes.data if a is not None else None


def version():
    return lib().rfmf_version().decode()


def parse_gset(text, forced_scale=0.0):
    """Gset/MQLib text (str, bytes or a path) -> dict(n=header N, u, v, w,
    scale, zero_dropped) with the reference reader's rules (rfmf_gset_parse)."""
    import os
    if isinstance(text, (str, os.PathLike)) and os.path.exists(str(text)):
        with open(text, "rb") as f:
            data = f.read()
    else:
        data = text.encode() if isinstance(text, str) else bytes(text)
    N, M = ct.c_int64(), ct.c_int64()
    check(lib().rfmf_gset_header(data, len(data), ct.byref(N), ct.byref(M)))
    cap = max(M.value, 1)
    u = np.zeros(cap, np.int64)
    v = np.zeros(cap, np.int64)
    w = np.zeros(cap, np.int64)
    k, scale, dropped = ct.c_int64(), ct.c_double(), ct.c_int64()
    check(lib().rfmf_gset_parse(data, len(data), float(forced_scale), cap, _p(u), _p(v), _p(w),
                                ct.byref(k), ct.byref(scale), ct.byref(dropped)))
    return dict(n=N.value, u=u[:k.value], v=v[:k.value], w=w[:k.value], scale=scale.value,
                zero_dropped=dropped.value)


def initial_spins(seed, n):
    """Chain's initial spins from its RAW seed (src/host_common.cpp:40-45)."""
    out = np.zeros(n, np.int8)
    lib().rfmf_initial_spins(int(seed) % 2**64, n, _p(out))
    return out


def total_steps(iters):
    it = np.ascontiguousarray(iters, np.uint64)
    r = lib().rfmf_total_steps(len(it), _p(it))
    if r < 0:
        raise RfmfError(4, "iters total more than 10^12 sweeps")
    return r


def beta_fixed(step, t0):
    return lib().rfmf_beta_fixed(int(step), float(t0))


def score_safe_int32(total, t0, B):
    return bool(lib().rfmf_score_safe_int32(int(total), float(t0), int(B)))


def max_weighted_degree(g):
    return lib().rfmf_max_weighted_degree(g.n, _p(g.offsets), _p(g.weight))


def cut_value(g, spin):
    spin = np.ascontiguousarray(spin, np.int8)
    return lib().rfmf_cut_value(g.n, _p(g.offsets), _p(g.col), _p(g.weight), _p(spin))


def beta_tables(t0s, total):
    """buildBetaRunTables: returns (run_end int64, run_val int32, chain_off)."""
    t = np.ascontiguousarray(t0s, np.float64)
    runs = ct.c_int64(0)
    off = np.zeros(len(t), np.int64)
    check(lib().rfmf_beta_tables(_p(t), len(t), int(total), None, None, _p(off), 0,
                                 ct.byref(runs)))
    end = np.zeros(runs.value, np.int64)
    val = np.zeros(runs.value, np.int32)
    check(lib().rfmf_beta_tables(_p(t), len(t), int(total), _p(end), _p(val), _p(off),
                                 runs.value, ct.byref(runs)))
    return end, val, off


def make_config(threads_per_chain=0, score_path=0, chains_per_cta=0, csr_format=0,
                gain_width=0, corr=0, s_width=32, device=0):
    """rfmf_launch_config; 0 everywhere = autotuned.  csr_format: 1 unit16,
    2 packed32 (shared memory), 3 HBM (most compact entries), 4 HBM 8-byte
    entries; gain_width: 1 (int8) or 4 (int32)."""
    c = LaunchConfig()
    c.corr = corr
    c.device = device
    c.s_width = s_width
    c.threads_per_chain = threads_per_chain
    c.score_path = score_path
    c.chains_per_cta = chains_per_cta
    c.csr_format = csr_format
    c.gain_width = gain_width
    return c


class Context:
    """One CUDA device + stream (rfmf_context)."""

    def __init__(self, device=0):
        h = ct.c_void_p()
        check(lib().rfmf_context_create(device, ct.byref(h)))
        self.h = h
        self.device = device

    def info(self):
        sms, smem = ct.c_int(0), ct.c_int(0)
        check(lib().rfmf_context_info(self.h, ct.byref(sms), ct.byref(smem)))
        return dict(sm_count=sms.value, smem_optin=smem.value)

    def stream(self):
        """The context's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        p = ct.c_void_p()
        check(lib().rfmf_context_stream(self.h, ct.byref(p)))
        return p.value or 0

    def beta_cache(self):
        """Device-resident beta tables of the context: live tables, their
        bytes, and uploads so far."""
        t, b, u = ct.c_int64(), ct.c_int64(), ct.c_uint64()
        check(lib().rfmf_context_beta_cache(self.h, ct.byref(t), ct.byref(b), ct.byref(u)))
        return dict(tables=t.value, device_bytes=b.value, uploads=u.value)

    def close(self):
        if self.h:
            lib().rfmf_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceGraph:
    """A CSR graph resident in device memory (rfmf_graph)."""

    def __init__(self, ctx, g):
        h = ct.c_void_p()
        self.off = np.ascontiguousarray(g.offsets, np.uint32)
        self.col = np.ascontiguousarray(g.col, np.int32)
        self.w = np.ascontiguousarray(g.weight, np.int32)
        check(lib().rfmf_graph_create(ctx.h, g.n, _p(self.off), _p(self.col), _p(self.w),
                                      ct.byref(h)))
        self.h = h
        self.ctx = ctx
        self.g = g
        self.n = g.n

    @classmethod
    def from_edges(cls, ctx, u, v, w):
        """Graph built on the device from an edge list (rfmf_graph_from_edges):
        duplicates keep their first weight, ids renumbered densely in
        ascending order, rows sorted."""
        self = cls.__new__(cls)
        uu = np.ascontiguousarray(u, np.int64)
        vv = np.ascontiguousarray(v, np.int64)
        ww = np.ascontiguousarray(w, np.int64)
        h = ct.c_void_p()
        n = ct.c_int64()
        check(lib().rfmf_graph_from_edges(ctx.h, len(uu), _p(uu), _p(vv), _p(ww), ct.byref(h),
                                          ct.byref(n)))
        self.h = h
        self.ctx = ctx
        self.g = None
        self.n = n.value
        return self

    def info(self):
        n, m, B = ct.c_int64(), ct.c_int64(), ct.c_int64()
        check(lib().rfmf_graph_info(self.h, ct.byref(n), ct.byref(m), ct.byref(B)))
        return dict(n=n.value, m=m.value, max_weighted_degree=B.value)

    def csr(self):
        """(offsets, col, weight) copied back from the device."""
        m = self.info()["m"]
        off = np.zeros(self.n + 1, np.uint32)
        col = np.zeros(2 * m, np.int32)
        w = np.zeros(2 * m, np.int32)
        check(lib().rfmf_graph_csr(self.h, _p(off), _p(col), _p(w)))
        return off, col, w

    def orig_ids(self):
        out = np.zeros(self.n, np.int64)
        check(lib().rfmf_graph_orig_ids(self.h, _p(out)))
        return out

    def close(self):
        if self.h:
            lib().rfmf_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class AnnealResult:
    end_spins: np.ndarray
    best_spins: np.ndarray
    kernel_ms: float
    best_vals: np.ndarray
    final_vals: np.ndarray


def anneal_gpu(ctx, dgraph, max_weighted_deg, initial_spins_, t0s, phases, iters, solver_seeds,
               cfg=None):
    """gpu3::annealGpu: C chains over one graph, host buffers in and out."""
    spins = np.ascontiguousarray(initial_spins_, np.int8)
    C = spins.shape[0]
    n = dgraph.n
    assert spins.shape == (C, n)
    t = np.ascontiguousarray(t0s, np.float64)
    ph = np.ascontiguousarray(phases, np.uint64)
    it = np.ascontiguousarray(iters, np.uint64)
    sd = np.array([int(s) % 2**64 for s in solver_seeds], np.uint64)
    assert len(t) == C and len(sd) == C and len(ph) == len(it)
    end = np.zeros((C, n), np.int8)
    best = np.zeros((C, n), np.int8)
    bv = np.zeros(C, np.int64)
    fv = np.zeros(C, np.int64)
    ms = ct.c_float(0)
    cfg = cfg or make_config()
    check(lib().rfmf_anneal(ctx.h, dgraph.h, int(max_weighted_deg), C, _p(spins), _p(t),
                            len(ph), _p(ph), _p(it), _p(sd), ct.byref(cfg), _p(end), _p(best),
                            ct.byref(ms), _p(bv), _p(fv)))
    return AnnealResult(end, best, ms.value, bv, fv)


def autotune(ctx, dgraphs, t0s, solver_seeds, init_spins, phases, iters, trial_sweeps=0,
             base=None):
    """rfmf_autotune: time candidate launch plans on short trial batches of
    these chains; returns (best config, [(candidate config, us per
    chain-sweep), ...]).  Cached in the context by batch shape."""
    C = len(dgraphs)
    garr = (ct.c_void_p * C)(*[g.h.value for g in dgraphs])
    t = np.ascontiguousarray(t0s, np.float64)
    sd = np.array([int(s) % 2**64 for s in solver_seeds], np.uint64)
    flat = np.ascontiguousarray(np.concatenate([np.asarray(s, np.int8) for s in init_spins]))
    ph = np.ascontiguousarray(phases, np.uint64)
    it = np.ascontiguousarray(iters, np.uint64)
    best = LaunchConfig()
    n = ct.c_int(16)
    cands = (LaunchConfig * 16)()
    us = np.zeros(16, np.float32)
    check(lib().rfmf_autotune(ctx.h, C, garr, _p(t), _p(sd), _p(flat), len(ph), _p(ph), _p(it),
                              int(trial_sweeps), ct.byref(base) if base is not None else None,
                              ct.byref(best), ct.byref(n), cands, _p(us)))
    return best, [(cands[k], float(us[k])) for k in range(min(n.value, 16))]


def debug_fail_host_alloc(countdown):
    """Testing aid: the countdown-th host allocation checkpoint from now on
    fails as if out of memory (rfmf_debug_fail_host_alloc); 0 disarms."""
    check(lib().rfmf_debug_fail_host_alloc(int(countdown)))


def debug_plan_items(chains, max_chains_per_cta, warps, level_ns, slots):
    """Testing aid: the batch planner's item sizes for one launch class on
    given costs (rfmf_debug_plan_items).  chains[q]: graph q's chains;
    level_ns[q][l - 1]: its item time per sweep at scheduler level l.
    Returns the chains per item of each graph."""
    G = len(chains)
    ch = np.ascontiguousarray(chains, np.int64)
    ns = np.ascontiguousarray(level_ns, np.float64).reshape(G, -1)
    out = np.zeros(G, np.int32)
    check(lib().rfmf_debug_plan_items(G, _p(ch), int(max_chains_per_cta), int(warps), _p(ns),
                                      int(slots), _p(out)))
    return [int(x) for x in out]


class Batch:
    """Chains over many graphs with device-resident state (rfmf_batch)."""

    @classmethod
    def restore(cls, ctx, dgraphs, t0s, solver_seeds, phases, iters, state, cfg=None):
        """A batch resumed from saved state: `state` is what read() returned
        (end_spins, best_spins, cur_vals, best_vals, sweeps_done)."""
        self = cls.__new__(cls)
        C = len(dgraphs)
        self.C = C
        self.ns = [g.n for g in dgraphs]
        self.ctx = ctx
        self.dgraphs = list(dgraphs)
        garr = (ct.c_void_p * C)(*[g.h.value for g in dgraphs])
        t = np.ascontiguousarray(t0s, np.float64)
        sd = np.array([int(s) % 2**64 for s in solver_seeds], np.uint64)
        end = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int8) for x in state["end_spins"]]))
        best = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int8) for x in state["best_spins"]]))
        cur = np.ascontiguousarray(state["cur_vals"], np.int64)
        bv = np.ascontiguousarray(state["best_vals"], np.int64)
        done = np.ascontiguousarray(state["sweeps_done"], np.uint64)
        ph = np.ascontiguousarray(phases, np.uint64)
        it = np.ascontiguousarray(iters, np.uint64)
        cfg = cfg or make_config()
        h = ct.c_void_p()
        check(lib().rfmf_batch_restore(ctx.h, C, garr, _p(t), _p(sd), len(ph), _p(ph), _p(it),
                                       ct.byref(cfg), _p(end), _p(best), _p(cur), _p(bv), _p(done),
                                       ct.byref(h)))
        self.h = h
        return self

    def __init__(self, ctx, dgraphs, t0s, solver_seeds, init_spins, phases, iters, cfg=None):
        C = len(dgraphs)
        self.C = C
        self.ns = [g.n for g in dgraphs]
        self.ctx = ctx
        self.dgraphs = list(dgraphs)   # keep alive
        garr = (ct.c_void_p * C)(*[g.h.value for g in dgraphs])
        t = np.ascontiguousarray(t0s, np.float64)
        sd = np.array([int(s) % 2**64 for s in solver_seeds], np.uint64)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(s, np.int8) for s in init_spins]))
        assert len(flat) == sum(self.ns)
        ph = np.ascontiguousarray(phases, np.uint64)
        it = np.ascontiguousarray(iters, np.uint64)
        cfg = cfg or make_config()
        h = ct.c_void_p()
        check(lib().rfmf_batch_create(ctx.h, C, garr, _p(t), _p(sd), _p(flat), len(ph),
                                      _p(ph), _p(it), ct.byref(cfg), ct.byref(h)))
        self.h = h

    def info(self):
        p = BatchPlan()
        check(lib().rfmf_batch_info(self.h, ct.byref(p)))
        return {name: getattr(p, name) for name, _ in BatchPlan._fields_}

    def run(self, sweeps):
        check(lib().rfmf_batch_run(self.h, int(sweeps)))

    def run_graph(self, sweeps, launches=1, replays=1):
        check(lib().rfmf_batch_run_graph(self.h, int(sweeps), int(launches), int(replays)))

    def run_timed(self, sweeps):
        """Launch, wait, and return the launch's device time in ms."""
        ms = ct.c_float(0)
        check(lib().rfmf_batch_run_timed(self.h, int(sweeps), ct.byref(ms)))
        return ms.value

    def improved_sweeps(self):
        out = np.zeros(self.C, np.uint64)
        check(lib().rfmf_batch_stats(self.h, _p(out)))
        return out

    def debug_set_cut(self, chain, cut):
        """Testing aid: overwrite a chain's carried cut on the device."""
        check(lib().rfmf_batch_debug_set_cut(self.h, int(chain), int(cut)))

    def synchronize(self):
        check(lib().rfmf_batch_synchronize(self.h))

    def read(self):
        tot = sum(self.ns)
        end = np.zeros(tot, np.int8)
        best = np.zeros(tot, np.int8)
        cur = np.zeros(self.C, np.int64)
        bv = np.zeros(self.C, np.int64)
        done = np.zeros(self.C, np.uint64)
        check(lib().rfmf_batch_read(self.h, _p(end), _p(best), _p(cur), _p(bv), _p(done)))
        splits = np.cumsum(self.ns)[:-1]
        return dict(end_spins=np.split(end, splits), best_spins=np.split(best, splits),
                    cur_vals=cur, best_vals=bv, sweeps_done=done)

    def cuts(self, best=False):
        """Cut of every chain's end (or best) spins, recomputed on the device."""
        out = np.zeros(self.C, np.int64)
        check(lib().rfmf_batch_cuts(self.h, 1 if best else 0, _p(out)))
        return out

    def partitions(self, best=False):
        """Partition strings ('0'/'1' per vertex) of every chain, built on the device."""
        stride = max(self.ns)
        buf = ct.create_string_buffer(self.C * stride)
        check(lib().rfmf_batch_partitions(self.h, 1 if best else 0, buf, stride))
        raw = buf.raw
        return [raw[c * stride:c * stride + n].decode() for c, n in enumerate(self.ns)]

    def best_vals(self):
        """Best cut of every chain so far (waits for launches in flight)."""
        bv = np.zeros(self.C, np.int64)
        check(lib().rfmf_batch_read(self.h, None, None, None, _p(bv), None))
        return bv

    def close(self):
        if self.h:
            lib().rfmf_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request server (rfmf_server): continuous batching of annealGpu-sized
    requests over persistent launches; submit from any thread, poll or wait,
    then take the results.  Each request's results equal anneal_gpu on the
    same inputs."""

    def __init__(self, ctx, window_sweeps=4096, max_chains=0, cfg=None, max_device_bytes=0):
        sc = ServerConfig()
        sc.window_sweeps = int(window_sweeps)
        sc.max_chains = int(max_chains)
        sc.launch = cfg or make_config()
        sc.max_device_bytes = int(max_device_bytes)
        h = ct.c_void_p()
        check(lib().rfmf_server_create(ctx.h, ct.byref(sc), ct.byref(h)))
        self.h = h
        self.ctx = ctx
        self._req = {}   # id -> (n, C, graph kept alive)

    def submit(self, dgraph, init_spins, t0s, phases, iters, solver_seeds):
        spins = np.ascontiguousarray(init_spins, np.int8)
        C = spins.shape[0]
        t = np.ascontiguousarray(t0s, np.float64)
        sd = np.array([int(s) % 2**64 for s in solver_seeds], np.uint64)
        ph = np.ascontiguousarray(phases, np.uint64)
        it = np.ascontiguousarray(iters, np.uint64)
        rid = ct.c_uint64()
        check(lib().rfmf_submit(self.h, dgraph.h, C, _p(spins), _p(t), len(ph), _p(ph), _p(it),
                                _p(sd), ct.byref(rid)))
        self._req[rid.value] = (dgraph.n, C, dgraph)
        return rid.value

    @staticmethod
    def _status(st):
        return dict(state=REQUEST_STATES[st.state], error=st.error, sweeps_done=st.sweeps_done,
                    sweeps_total=st.sweeps_total, submit_s=st.submit_s, start_s=st.start_s,
                    finish_s=st.finish_s)

    def poll(self, rid):
        st = RequestStatus()
        check(lib().rfmf_poll(self.h, int(rid), ct.byref(st)))
        return self._status(st)

    def wait(self, rid, timeout=-1.0):
        st = RequestStatus()
        check(lib().rfmf_wait(self.h, int(rid), float(timeout), ct.byref(st)))
        return self._status(st)

    def result(self, rid):
        """Results of a done request (releases it); raises while it runs."""
        n, C, _ = self._req[rid]
        end = np.zeros((C, n), np.int8)
        best = np.zeros((C, n), np.int8)
        bv = np.zeros(C, np.int64)
        fv = np.zeros(C, np.int64)
        finished = self.poll(rid)["state"] in ("done", "failed", "cancelled")
        try:
            check(lib().rfmf_result(self.h, int(rid), _p(end), _p(best), _p(bv), _p(fv)))
        finally:
            if finished:
                self._req.pop(rid, None)
        return AnnealResult(end, best, 0.0, bv, fv)

    def cancel(self, rid):
        """Cancel a queued or running request (rfmf_cancel)."""
        check(lib().rfmf_cancel(self.h, int(rid)))

    def stats(self):
        s = ServerStats()
        check(lib().rfmf_server_stats_get(self.h, ct.byref(s)))
        return {name: getattr(s, name) for name, _ in ServerStats._fields_}

    def close(self):
        if self.h:
            lib().rfmf_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
