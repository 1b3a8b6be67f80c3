"""Request server (rfmf_submit / rfmf_poll / rfmf_wait / rfmf_result).

Every request's results must equal a standalone anneal_gpu of the same inputs
bit for bit (spins, best spins, best and final cuts), whatever shares its
launch windows: requests on different graphs, schedules, gain widths and
score paths, admitted at different window boundaries."""
import threading

import numpy as np
import pytest

from conftest import chains_for

pytestmark = pytest.mark.gpu


def _request(rfmf, g, seeds, t0s, phases, iters):
    init, solver = chains_for(g, seeds)
    return dict(g=g, init=init, solver=solver, t0s=t0s, phases=phases, iters=iters)


def _standalone(rfmf, ctx, dg, r):
    return rfmf.anneal_gpu(ctx, dg, r["g"].max_weighted_degree(), r["init"], r["t0s"],
                           r["phases"], r["iters"], r["solver"])


def _same(a, b):
    assert np.array_equal(a.end_spins, b.end_spins)
    assert np.array_equal(a.best_spins, b.best_spins)
    assert np.array_equal(a.best_vals, b.best_vals)
    assert np.array_equal(a.final_vals, b.final_vals)


def test_server_requests_match_standalone(rfmf, ctx):
    er = rfmf.erdos_renyi(600, 0.03, signed=True, seed=3)
    tor = rfmf.torus(20, 30, signed=True, seed=4)
    tree = rfmf.random_tree(900, seed=5)
    heavy = rfmf.erdos_renyi(300, 0.05, signed=True, seed=6)
    heavy.weight = heavy.weight * 9            # B > 127: int32 gains
    reqs = [
        _request(rfmf, er, list(range(40)), [35.0, 70.0, 140.0, 400.0] * 10,
                 [128, 16, 2, 1], [300, 300, 300, 300]),
        _request(rfmf, tor, list(range(100, 124)), [50.0] * 24, [64, 8, 1], [500, 500, 500]),
        _request(rfmf, tree, list(range(200, 216)), [100.0] * 16, [32, 0, 4], [700, 50, 700]),
        _request(rfmf, heavy, list(range(300, 310)), [35.0] * 10, [8, 1], [400, 400]),
        # tiny t0: the int64 score path
        _request(rfmf, er, list(range(400, 408)), [0.004] * 8, [16, 1], [200, 200]),
    ]
    dgs = {}
    for r in reqs:
        dgs.setdefault(id(r["g"]), rfmf.DeviceGraph(ctx, r["g"]))
    srv = rfmf.Server(ctx, window_sweeps=257)
    ids = []
    for r in reqs[:3]:
        ids.append(srv.submit(dgs[id(r["g"])], r["init"], r["t0s"], r["phases"], r["iters"], r["solver"]))
    srv.wait(ids[0], timeout=120)
    for r in reqs[3:]:   # join mid-flight
        ids.append(srv.submit(dgs[id(r["g"])], r["init"], r["t0s"], r["phases"], r["iters"], r["solver"]))
    for rid, r in zip(ids, reqs):
        st = srv.wait(rid, timeout=300)
        assert st["state"] == "done", st
        assert st["sweeps_done"] == st["sweeps_total"] == sum(i for p, i in zip(r["phases"], r["iters"]) if p)
        assert st["submit_s"] <= st["start_s"] <= st["finish_s"]
        _same(srv.result(rid), _standalone(rfmf, ctx, dgs[id(r["g"])], r))
    stats = srv.stats()
    assert stats["windows"] >= 6 and stats["launches"] > stats["windows"]   # several launch classes
    assert stats["queued"] == stats["running"] == stats["done"] == 0
    srv.close()


def test_server_admission_limit_and_threads(rfmf, ctx):
    g = rfmf.erdos_renyi(400, 0.04, signed=True, seed=8)
    dg = rfmf.DeviceGraph(ctx, g)
    srv = rfmf.Server(ctx, window_sweeps=500, max_chains=48)
    reqs = [_request(rfmf, g, list(range(1000 + 32 * k, 1032 + 32 * k)), [35.0 + k] * 32,
                     [32, 1], [600, 600]) for k in range(4)]
    ids = [None] * 4

    def sub(k):
        r = reqs[k]
        ids[k] = srv.submit(dg, r["init"], r["t0s"], r["phases"], r["iters"], r["solver"])

    th = [threading.Thread(target=sub, args=(k,)) for k in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    sts = [srv.wait(rid, timeout=300) for rid in ids]
    # 48 admitted chains: one 32-chain request at a time
    spans = sorted((s["start_s"], s["finish_s"]) for s in sts)
    for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
        assert b0 >= a1 - 1e-9
    for rid, r in zip(ids, reqs):
        _same(srv.result(rid), _standalone(rfmf, ctx, dg, r))
    srv.close()


def test_server_errors(rfmf, ctx):
    g = rfmf.torus(8, 8, signed=True, seed=1)
    dg = rfmf.DeviceGraph(ctx, g)
    srv = rfmf.Server(ctx, window_sweeps=100, max_chains=16)
    init, solver = chains_for(g, [1, 2])
    with pytest.raises(rfmf.RfmfError) as ei:
        srv.submit(dg, init, [35.0, -1.0], [1], [10], solver)
    assert ei.value.code == 1
    big, bsolver = chains_for(g, list(range(17)))
    with pytest.raises(rfmf.RfmfError) as ei:
        srv.submit(dg, big, [35.0] * 17, [1], [10], bsolver)
    assert ei.value.code == 4
    with pytest.raises(rfmf.RfmfError):
        srv.poll(987654321)
    rid = srv.submit(dg, init, [35.0, 40.0], [4, 1], [20000, 20000], solver)
    with pytest.raises(rfmf.RfmfError):
        srv.result(rid)              # not done yet (40000 sweeps, windows of 100)
    st = srv.wait(rid, timeout=300)
    assert st["state"] == "done"
    srv.result(rid)
    srv.close()


def test_shared_beta_tables_and_refusal_at_submit(rfmf, ctx):
    """Requests sharing a t0 ladder and length reuse one set of run tables
    (built on the submitting thread) and still equal standalone anneals; a
    schedule whose beta would overflow int32 is refused by rfmf_submit itself,
    before any device state, as rfmf_anneal refuses it."""
    g = rfmf.erdos_renyi(400, 0.04, signed=True, seed=8)
    dg = rfmf.DeviceGraph(ctx, g)
    ladder = [35.0, 50.0, 70.0, 100.0]
    reqs = [_request(rfmf, g, list(range(500 + 20 * k, 512 + 20 * k)), ladder * 3, [32, 4, 1],
                     [400, 400, 400]) for k in range(3)]
    srv = rfmf.Server(ctx, window_sweeps=300)
    ids = [srv.submit(dg, r["init"], r["t0s"], r["phases"], r["iters"], r["solver"]) for r in reqs]
    for rid, r in zip(ids, reqs):
        st = srv.wait(rid, timeout=300)
        assert st["state"] == "done", st
        _same(srv.result(rid), _standalone(rfmf, ctx, dg, r))
    bad = _request(rfmf, g, [1, 2], [1e-9, 35.0], [8, 1], [10**6, 10**6])
    with pytest.raises(rfmf.RfmfError):
        srv.submit(dg, bad["init"], bad["t0s"], bad["phases"], bad["iters"], bad["solver"])
    srv.close()


def test_server_device_byte_budget(rfmf, ctx):
    """max_device_bytes: each request's own device state here is 20,832 bytes
    (2 x 32 chains x 13 spin words, 1,200 beta runs x 12 bytes, two 16-byte
    schedule buffers, 32 chain records x 96 bytes), so under a 30,000-byte
    budget the requests run one at a time, and each still equals its
    standalone anneal; a request whose state alone exceeds the budget (two t0
    tables: 35,232 bytes) is refused at submission."""
    g = rfmf.erdos_renyi(400, 0.04, signed=True, seed=8)
    dg = rfmf.DeviceGraph(ctx, g)
    srv = rfmf.Server(ctx, window_sweeps=500, max_device_bytes=30000)
    reqs = [_request(rfmf, g, list(range(2000 + 32 * k, 2032 + 32 * k)), [35.0 + k] * 32,
                     [32, 1], [600, 600]) for k in range(3)]
    ids = [srv.submit(dg, r["init"], r["t0s"], r["phases"], r["iters"], r["solver"]) for r in reqs]
    sts = [srv.wait(rid, timeout=300) for rid in ids]
    spans = sorted((s["start_s"], s["finish_s"]) for s in sts)
    for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
        assert b0 >= a1 - 1e-9
    for rid, r in zip(ids, reqs):
        _same(srv.result(rid), _standalone(rfmf, ctx, dg, r))
    two = _request(rfmf, g, list(range(3000, 3032)), [35.0, 36.0] * 16, [32, 1], [600, 600])
    with pytest.raises(rfmf.RfmfError) as ei:
        srv.submit(dg, two["init"], two["t0s"], two["phases"], two["iters"], two["solver"])
    assert ei.value.code == 4
    srv.close()


def test_device_beta_tables_shared_within_a_context(rfmf, ctx):
    """Beta run tables live on the device once per (t0, sweeps) per context:
    a second batch, an rfmf_anneal call and a served request on the same
    ladder and length upload nothing more, while a new length uploads its
    own tables; every result still equals a standalone anneal (on another
    context, with its own tables)."""
    c = rfmf.Context(0)
    g = rfmf.erdos_renyi(400, 0.04, signed=True, seed=18)
    dg = rfmf.DeviceGraph(c, g)
    dref = rfmf.DeviceGraph(ctx, g)
    ladder = [35.0, 50.0, 70.0, 100.0, 140.0, 200.0, 280.0, 400.0]
    phases, iters = [32, 4, 1], [300, 300, 300]
    assert c.beta_cache()["uploads"] == 0
    r1 = _request(rfmf, g, list(range(900, 916)), ladder * 2, phases, iters)
    b1 = rfmf.Batch(c, [dg] * 16, r1["t0s"], r1["solver"], list(r1["init"]), phases, iters)
    assert c.beta_cache()["uploads"] == 8 and c.beta_cache()["tables"] == 8
    r2 = _request(rfmf, g, list(range(950, 966)), ladder * 2, phases, iters)
    b2 = rfmf.Batch(c, [dg] * 16, r2["t0s"], r2["solver"], list(r2["init"]), phases, iters)
    got = rfmf.anneal_gpu(c, dg, g.max_weighted_degree(), r1["init"], r1["t0s"], phases, iters,
                          r1["solver"])
    srv = rfmf.Server(c, window_sweeps=250)
    rid = srv.submit(dg, r2["init"], r2["t0s"], phases, iters, r2["solver"])
    assert srv.wait(rid, timeout=300)["state"] == "done"
    served = srv.result(rid)
    srv.close()
    assert c.beta_cache()["uploads"] == 8
    for b in (b1, b2):
        b.run(sum(iters))
    o1, o2 = b1.read(), b2.read()
    b1.close()
    b2.close()
    ref1 = _standalone(rfmf, ctx, dref, r1)
    ref2 = _standalone(rfmf, ctx, dref, r2)
    _same(got, ref1)
    _same(served, ref2)
    assert np.array_equal(np.stack(o1["best_spins"]), ref1.best_spins)
    assert np.array_equal(o1["best_vals"], ref1.best_vals)
    assert np.array_equal(np.stack(o2["end_spins"]), ref2.end_spins)
    assert np.array_equal(o2["cur_vals"], ref2.final_vals)
    # another length: its own tables
    got3 = rfmf.anneal_gpu(c, dg, g.max_weighted_degree(), r1["init"], r1["t0s"], phases,
                           [100, 100, 100], r1["solver"])
    assert c.beta_cache()["uploads"] == 16
    _same(got3, rfmf.anneal_gpu(ctx, dref, g.max_weighted_degree(), r1["init"], r1["t0s"], phases,
                                [100, 100, 100], r1["solver"]))
    dg.close()
    dref.close()
    c.close()


def test_cancel_queued_and_running_requests(rfmf, ctx):
    """rfmf_cancel: a queued request is cancelled at once and never starts; a
    running one leaves at a window boundary, freeing its chains for the next
    request; the others still equal their standalone anneals, and the
    cancelled ones' results are refused."""
    g = rfmf.erdos_renyi(500, 0.03, signed=True, seed=28)
    dg = rfmf.DeviceGraph(ctx, g)
    srv = rfmf.Server(ctx, window_sweeps=200, max_chains=64)
    long_ = _request(rfmf, g, list(range(3100, 3164)), [35.0] * 64, [16, 1], [10**6, 10**6])
    queued = _request(rfmf, g, list(range(3200, 3232)), [50.0] * 32, [8, 1], [400, 400])
    short = _request(rfmf, g, list(range(3300, 3332)), [70.0] * 32, [8, 1], [400, 400])
    ids = [srv.submit(dg, r["init"], r["t0s"], r["phases"], r["iters"], r["solver"])
           for r in (long_, queued, short)]
    import time
    t_end = time.time() + 60
    while srv.poll(ids[0])["state"] != "running" and time.time() < t_end:
        time.sleep(0.01)
    assert srv.poll(ids[0])["state"] == "running"
    assert srv.poll(ids[1])["state"] == "queued"        # max_chains: 64 running
    srv.cancel(ids[1])
    st1 = srv.poll(ids[1])
    assert st1["state"] == "cancelled" and st1["start_s"] == 0.0
    srv.cancel(ids[0])
    st0 = srv.wait(ids[0], timeout=120)
    assert st0["state"] == "cancelled" and st0["sweeps_done"] < st0["sweeps_total"]
    st2 = srv.wait(ids[2], timeout=300)
    assert st2["state"] == "done"
    _same(srv.result(ids[2]), _standalone(rfmf, ctx, dg, short))
    for rid in ids[:2]:
        with pytest.raises(rfmf.RfmfError):
            srv.result(rid)
    stats = srv.stats()
    assert stats["queued"] == stats["running"] == 0
    srv.close()


def test_injected_host_allocation_failure_fails_one_request(rfmf, ctx):
    """A host allocation failure while the worker admits a request fails that
    request with RFMF_ERR_NOMEM (it is not lost: rfmf_wait returns); the
    server keeps serving and the next request equals its standalone anneal.
    The failure is injected on the host (rfmf_debug_fail_host_alloc), no GPU
    fault is involved."""
    g = rfmf.erdos_renyi(300, 0.04, signed=True, seed=29)
    dg = rfmf.DeviceGraph(ctx, g)
    srv = rfmf.Server(ctx, window_sweeps=300)
    a = _request(rfmf, g, list(range(3400, 3408)), [35.0] * 8, [8, 1], [300, 300])
    b = _request(rfmf, g, list(range(3500, 3508)), [50.0] * 8, [8, 1], [300, 300])
    c = _request(rfmf, g, list(range(3600, 3608)), [70.0] * 8, [8, 1], [300, 300])
    ra = srv.submit(dg, a["init"], a["t0s"], a["phases"], a["iters"], a["solver"])
    assert srv.wait(ra, timeout=120)["state"] == "done"
    _same(srv.result(ra), _standalone(rfmf, ctx, dg, a))
    # checkpoint 1: rfmf_submit of b; checkpoint 2: b's admission in the worker
    rfmf.debug_fail_host_alloc(2)
    rb = srv.submit(dg, b["init"], b["t0s"], b["phases"], b["iters"], b["solver"])
    stb = srv.wait(rb, timeout=120)
    rfmf.debug_fail_host_alloc(0)
    assert stb["state"] == "failed" and stb["error"] == 3, stb
    with pytest.raises(rfmf.RfmfError) as ei:
        srv.result(rb)
    assert ei.value.code == 3
    rc_ = srv.submit(dg, c["init"], c["t0s"], c["phases"], c["iters"], c["solver"])
    assert srv.wait(rc_, timeout=120)["state"] == "done"
    _same(srv.result(rc_), _standalone(rfmf, ctx, dg, c))
    # a batch whose creation meets the failure reports it and nothing leaks
    rfmf.debug_fail_host_alloc(1)
    with pytest.raises(rfmf.RfmfError) as ei:
        rfmf.Batch(ctx, [dg] * 8, c["t0s"], c["solver"], list(c["init"]), c["phases"], c["iters"])
    rfmf.debug_fail_host_alloc(0)
    assert ei.value.code == 3
    srv.close()
