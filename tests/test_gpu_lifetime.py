"""Destroy order.  A context's handle may be released before the graphs,
batches and servers made on it (a garbage collector finalises objects in
its own order, e.g. at interpreter exit when module globals sit in a
reference cycle); the context then lives until the last of them is
destroyed, and they keep working meanwhile."""
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from conftest import ROOT, chains_for

pytestmark = pytest.mark.gpu


def test_objects_outlive_the_context_handle(rfmf, oracle):
    ctx = rfmf.Context(0)
    g = rfmf.erdos_renyi(200, 0.05, signed=True, seed=1)
    dg = rfmf.DeviceGraph(ctx, g)
    init, solver = chains_for(g, [1, 2, 3, 4])
    t0s, phases, iters = [50.0, 70.0, 100.0, 140.0], [4, 1], [60, 60]
    b = rfmf.Batch(ctx, [dg] * 4, t0s, solver, list(init), phases, iters)
    srv = rfmf.Server(ctx, window_sweeps=40)
    ctx.close()                       # the caller's handle goes first
    b.run(120)
    r = b.read()
    rid = srv.submit(dg, init, t0s, phases, iters, solver)
    assert srv.wait(rid, 60.0)["state"] == "done"
    s = srv.result(rid)
    ref = oracle.anneal(g, init, t0s, solver, phases, iters)
    assert np.array_equal(np.stack(r["best_spins"]), ref["best_spins"])
    assert np.array_equal(s.best_spins, ref["best_spins"])
    dg.close()                        # then the graph, before the batch and server using it
    b.close()
    srv.close()


def test_interpreter_exit_finalises_in_any_order(tmp_path):
    """A script that leaves a context, graph, batch and server open, with a
    module-level function (the module's globals are then collected as a
    cycle, finalisers in arbitrary order), exits cleanly."""
    script = tmp_path / "leave_open.py"
    script.write_text(textwrap.dedent(f"""
        import sys
        sys.path.insert(0, {str(ROOT)!r})
        import rfmf_gb300 as R
        ctx = R.Context(0)
        g = R.erdos_renyi(300, 0.04, signed=True, seed=2)
        dg = R.DeviceGraph(ctx, g)
        init = [R.initial_spins(s, g.n) for s in range(8)]
        sol = [R.solver_seed(s) for s in range(8)]
        b = R.Batch(ctx, [dg] * 8, [60.0] * 8, sol, init, [8, 1], [100, 100])
        b.run(200)
        srv = R.Server(ctx, window_sweeps=50)
        rid = srv.submit(dg, init, [60.0] * 8, [8, 1], [100, 100], sol)
        srv.wait(rid, 60.0)

        def helper():
            return ctx, dg, b, srv

        print("ok", int(b.best_vals().max()) > 0)
    """))
    r = subprocess.run([sys.executable, str(script)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
    assert r.stdout.strip() == "ok True"
