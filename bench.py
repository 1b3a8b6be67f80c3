#!/usr/bin/env python3
"""bench.py -- chain-steps/s of the RFMF annealer on GB300.

Workload (the plain-method mid-size configuration): a 50x60 toroidal grid
(n=3000, 6000 edges, weights uniform +-1) and an Erdos-Renyi graph n=2000
with mean degree ~19 (weights uniform +-1), 1024 chains per graph (raw seeds
0..1023 per graph on rank 0), the reference's default schedule (phases
128,64,32,16,8,4,2,1 with equal sweeps per phase) and t0 ladder
35,50,70,100,140,200,280,400 assigned round-robin.  Synthetic seeded graphs
of those shapes stand in for the Gset instances.

One STEP is one rfmf_batch_run_timed window that advances all 2048 chains by
sweeps/steps sweeps (one persistent launch, or one per phase where the
window crosses a phase boundary: both graphs share a launch class, whose
work items are sized per phase); the K timed steps together are one
complete anneal of --sweeps sweeps per chain (default 10^7, the
configuration's budget), with the chain state resident on the device
between steps.  value = chains * sweeps / (sum of the K window times, CUDA
events on the library's stream).  The L2 is
flushed (256 MB write) between timed steps, outside the events.

e2e: the same metric through the public drop-in call (rfmf_graph_create +
rfmf_anneal, host buffers, synchronous) on the same graphs and chains with
sweeps/steps sweeps per chain per call, host<->device copies inside the
timed region.

--impl reference: the CPU restatement of the reference's sweep (oracle/,
there is no CPU annealer in the reference) on all host cores, on a bounded
sample of the same workload.
"""
import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

LADDER = [35.0, 50.0, 70.0, 100.0, 140.0, 200.0, 280.0, 400.0]
PHASES = [128, 64, 32, 16, 8, 4, 2, 1]
WORKLOAD = "torus50x60_pm1+er2000_d19_pm1"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# The large sparse shapes (100x200 torus, random tree n = 10000, ER n = 5000
# mean degree 5; 256 chains each): a profiling and parity workload whose
# CSRs do not all fit shared memory beside the chains (the HBM walk).
LARGE_WORKLOAD = "torus100x200_pm1+tree10000+er5000_d5_pm1"
WORKLOAD_CHAINS = {WORKLOAD: 1024, LARGE_WORKLOAD: 256}


def workload_graphs(name=WORKLOAD):
    import rfmf_gb300 as R
    if name == LARGE_WORKLOAD:
        return [R.torus(100, 200, signed=True, seed=0, name="torus100x200"),
                R.random_tree(10000, seed=0, name="tree10000"),
                R.erdos_renyi_sparse(5000, 5, signed=True, seed=0, name="er5000_d5")]
    return [R.torus(50, 60, signed=True, seed=0, name="torus50x60"),
            R.erdos_renyi_degree(2000, 19, signed=True, seed=0, name="er2000_d19")]


def chain_setup(graphs, chains_per_graph, seed_base):
    import rfmf_gb300 as R
    per = []
    for g in graphs:
        seeds = [seed_base + i for i in range(chains_per_graph)]
        per.append(dict(g=g, seeds=seeds,
                        init=np.stack([R.initial_spins(s, g.n) for s in seeds]),
                        solver=[R.solver_seed(s) for s in seeds],
                        t0s=[LADDER[i % 8] for i in range(chains_per_graph)]))
    return per


def schedule(sweeps, phases=None):
    phases = list(phases or PHASES)
    per = sweeps // len(phases)
    return phases, [per] * len(phases)


def sweep_bytes(n, m, P):
    """Algorithmic bytes of one chain-sweep (excluding best-spin copies):
    SELECT reads spin (1 B) + local field (4 B) per vertex; FLIP per winner
    reads an offsets pair (8 B), walks its row (8 B/entry) and updates each
    neighbour's field (8 B/entry)."""
    Pe = min(P, n)
    dbar = 2.0 * m / n
    return 5.0 * n + Pe * (8.0 + 16.0 * dbar)


def window_bytes(graphs_chains, phases, iters, s0, s1):
    """Sum of sweep_bytes over executed sweeps [s0, s1) for every chain."""
    tot = 0.0
    for g, nch in graphs_chains:
        acc = 0
        for P, it in zip(phases, iters):
            if P == 0:
                continue
            lo, hi = max(s0, acc), min(s1, acc + it)
            if hi > lo:
                tot += nch * (hi - lo) * sweep_bytes(g.n, g.m, P)
            acc += it
    return tot


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self, first_sample_timeout=30.0):
        """Start sampling and return once the first sample is written (NVML
        is initialised), so the sampler's start-up stays out of timed work."""
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
            return
        t_end = time.perf_counter() + first_sample_timeout
        while time.perf_counter() < t_end and self.p.poll() is None:
            if os.path.getsize(self.f.name) > 0:
                break
            time.sleep(0.05)

    def stop(self):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(", ") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip() == "Active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        load = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return {}
    return {}


def profile_traffic():
    """DRAM bytes per launch of the annealing kernel from a committed ncu
    summary (profiles/anneal_kernel_traffic.json), or None."""
    p = ROOT / "profiles" / "anneal_kernel_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return None
    return None


# --------------------------------------------------------------- CPU arms
SOLVER_SEED_OFFSET = 0xC2B2AE3D27D4EB4F


def _oracle():
    """The oracle (the C restatement of the reference's sweep): the CPU arms
    use its own initial spins and nothing of librfmf.so."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as ora
    ora.lib()
    return ora


def _cpu_chains(ora, g, seeds):
    init = np.stack([ora.initial_spins(s, g.n) for s in seeds])
    solver = [(int(s) + SOLVER_SEED_OFFSET) % 2**64 for s in seeds]
    return init, solver


def cpu_rate(graphs, steps, warmup, target_s, rank_seed_base=0):
    """Oracle on all host cores: one chain per core over a compressed schedule
    (same phases, equal sweeps per phase) on the workload's graphs.  Every
    step's inputs are built before the clock starts."""
    ora = _oracle()
    cores = ora.default_threads()
    # calibrate sweeps so one step takes ~target_s
    g0 = graphs[0]
    init1, sol1 = _cpu_chains(ora, g0, [1])
    t = time.perf_counter()
    ora.anneal(g0, init1, [35.0], sol1, PHASES, [40] * 8, nthreads=1)
    per_sweep = (time.perf_counter() - t) / 320 * (sum(g.n for g in graphs) / g0.n / len(graphs))
    # the two graphs run one after the other, each with one chain per core
    sweeps = max(800, int(target_s / 2 / max(per_sweep, 1e-7) / 8) * 8)
    nch = max(cores, 2)
    per_graph = [nch // 2, nch - nch // 2]
    inputs = []
    for step in range(warmup + steps):
        row = []
        for g, k in zip(graphs, per_graph):
            seeds = [rank_seed_base + 10000 * step + i for i in range(k)]
            init, solver = _cpu_chains(ora, g, seeds)
            row.append((g, k, init, solver, [LADDER[i % 8] for i in range(k)]))
        inputs.append(row)
    rates = []
    for step in range(warmup + steps):
        total_chain_sweeps = 0
        t = time.perf_counter()
        for g, k, init, solver, t0s in inputs[step]:
            ora.anneal(g, init, t0s, solver, PHASES, [sweeps // 8] * 8, nthreads=cores)
            total_chain_sweeps += k * sweeps
        el = time.perf_counter() - t
        if step >= warmup:
            rates.append((total_chain_sweeps, el))
    cs = sum(r[0] for r in rates)
    el = sum(r[1] for r in rates)
    sample = (f"{per_graph[0]}+{per_graph[1]} chains (torus50x60 + er2000_d19) x {sweeps} sweeps "
              f"(phases 128..1, {sweeps // 8} each) per step, {steps} step(s)")
    return cs / el, cores, sample, el


def cpu_config1(target_s):
    """The plain-method small case on the CPU restatement: ER n = 800, p = 0.06,
    +1 weights, 32 chains (raw seeds 0..31, t0 ladder), the default schedule
    compressed to a bounded sweep count, one chain per core."""
    import rfmf_gb300 as R
    ora = _oracle()
    cores = ora.default_threads()
    g = R.erdos_renyi(800, 0.06, seed=0, name="er800_p0.06")
    init, sol = _cpu_chains(ora, g, list(range(32)))
    t0s = [LADDER[i % 8] for i in range(32)]
    t = time.perf_counter()
    ora.anneal(g, init[:cores], t0s[:cores], sol[:cores], PHASES, [64] * 8, nthreads=cores)
    per = (time.perf_counter() - t) / (512 * max(1, min(cores, 32) // cores))
    sweeps = max(800, int(target_s / max(per, 1e-7) * cores / 32 / 8) * 8)
    t = time.perf_counter()
    ora.anneal(g, init, t0s, sol, PHASES, [sweeps // 8] * 8, nthreads=cores)
    el = time.perf_counter() - t
    return {"value": 32 * sweeps / el, "unit": "chain-steps/s", "cores": cores, "kind": "port",
            "sample": f"ER n=800 p=0.06 +1, 32 chains x {sweeps} sweeps (phases 128..1), "
                      f"{el:.1f} s"}


def gpu_config1(ctx):
    """The plain-method small case on the GPU through the drop-in call: ER
    n = 800, p = 0.06, +1 weights, 32 chains (raw seeds 0..31, t0 ladder),
    the default schedule at its full 10^6 sweeps; chain-steps over the
    call's device time, and over its wall time with host buffers."""
    import rfmf_gb300 as R
    g = R.erdos_renyi(800, 0.06, seed=0, name="er800_p0.06")
    dg = R.DeviceGraph(ctx, g)
    seeds = list(range(32))
    init = np.stack([R.initial_spins(s, g.n) for s in seeds])
    sol = [R.solver_seed(s) for s in seeds]
    t0s = [LADDER[i % 8] for i in range(32)]
    sweeps = 1_000_000
    t = time.perf_counter()
    res = R.anneal_gpu(ctx, dg, g.max_weighted_degree(), init, t0s, PHASES, [sweeps // 8] * 8, sol)
    wall = time.perf_counter() - t
    dg.close()
    return {"value": 32 * sweeps / (res.kernel_ms / 1e3), "unit": "chain-steps/s",
            "e2e_value": 32 * sweeps / wall, "best_cut": int(res.best_vals.max()),
            "sample": "ER n=800 p=0.06 +1, 32 chains x 10^6 sweeps (phases 128..1), rfmf_anneal"}


# --------------------------------------------------------------- GPU arm
def gpu_arm(args, rank, world):
    import torch

    import rfmf_gb300 as R
    R.lib(build_if_missing=True)
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    ctx = R.Context(dev)
    graphs = workload_graphs(args.workload)
    dgs = [R.DeviceGraph(ctx, g) for g in graphs]
    K, W = args.steps, args.warmup
    sweeps = args.sweeps
    main_phases = [int(x) for x in str(args.phases).split(",")] if args.phases else PHASES
    q = len(main_phases) * K
    if sweeps % q:
        sweeps = (sweeps // q) * q
    per_step = sweeps // K
    phases, iters = schedule(sweeps, main_phases)
    cfg = R.make_config(threads_per_chain=args.threads, chains_per_cta=args.chains_per_cta,
                        csr_format=args.csr_format)
    base = rank * args.chains
    setup = chain_setup(graphs, args.chains, base)
    tuned = None
    if not args.no_autotune:
        # measured plan: candidates timed on a compressed copy of the schedule
        gl_, ini_, sol_, t0_ = [], [], [], []
        for k, s_ in enumerate(setup):
            gl_ += [dgs[k]] * len(s_["seeds"])
            ini_ += list(s_["init"])
            sol_ += s_["solver"]
            t0_ += s_["t0s"]
        cfg, cands = R.autotune(ctx, gl_, t0_, sol_, ini_, phases, iters, base=cfg)
        tuned = {"chosen": {"threads_per_chain": cfg.threads_per_chain, "csr_format": cfg.csr_format},
                 "candidates": [{"threads_per_chain": c.threads_per_chain, "csr_format": c.csr_format,
                                 "us_per_chain_sweep": round(us, 5)} for c, us in cands],
                 "note": "0 = the planner's rule; csr_format 3 = HBM walks"}

    def batch_for(setup_, ph, it):
        gl, ini, sol, t0 = [], [], [], []
        for k, s in enumerate(setup_):
            gl += [dgs[k]] * len(s["seeds"])
            ini += list(s["init"])
            sol += s["solver"]
            t0 += s["t0s"]
        return R.Batch(ctx, gl, t0, sol, ini, ph, it, cfg)

    # warm-up: W launches of a separate anneal (different seeds), same sizes
    wsetup = chain_setup(graphs, args.chains, base + 1_000_000)
    wb = batch_for(wsetup, phases, iters)
    for _ in range(W):
        wb.run_timed(per_step)
    info = wb.info()
    wb.close()

    b = batch_for(setup, phases, iters)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    gc = [(g, args.chains) for g in graphs]
    clocks = ClockSampler(dev)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = b.info()["launches"]
    clocks.start()
    time.sleep(0.5)
    t_wall = time.perf_counter()
    step_ms, step_bytes, best_by_step = [], [], []
    imp_prev = np.zeros(len(graphs) * args.chains, np.uint64)
    for k in range(K):
        flush.zero_()
        torch.cuda.synchronize()
        ms = b.run_timed(per_step)
        step_ms.append(ms)
        imp = b.improved_sweeps()
        d_imp = (imp - imp_prev).astype(np.float64)
        imp_prev = imp
        ns = np.concatenate([[g.n] * args.chains for g in graphs])
        step_bytes.append(window_bytes(gc, phases, iters, k * per_step, (k + 1) * per_step) +
                          float(np.dot(ns, d_imp)))
        bv = b.best_vals()
        best_by_step.append([int(bv[i * args.chains:(i + 1) * args.chains].max())
                             for i in range(len(graphs))])
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    timed_launches = b.info()["launches"] - launches0
    total_ms = sum(step_ms)
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms = float(tt.item())
    out = b.read()
    done = out["sweeps_done"]
    assert all(int(d) == sweeps for d in done), "not every chain finished its schedule"
    chain_steps = len(graphs) * args.chains * sweeps
    value = chain_steps * world / (total_ms / 1e3)
    # consistency: kernel-tracked best == recompute of best spins (spot check)
    for i in (0, args.chains):
        g = graphs[i // args.chains]
        assert out["best_vals"][i] == g.cut_value(out["best_spins"][i])
    b.close()

    # time-to-target: target = each graph's best cut at the end of the anneal;
    # first step boundary at which the running best over its chains reaches it
    tt = []
    for i, g in enumerate(graphs):
        target = best_by_step[-1][i]
        k_hit = next(k for k in range(K) if best_by_step[k][i] >= target)
        tt.append({"graph": g.name, "target_cut": target, "sweeps": (k_hit + 1) * per_step,
                   "seconds": sum(step_ms[:k_hit + 1]) / 1e3})

    # the CPU-runnable small case, on the GPU (rank 0 of the default workload)
    config1 = (gpu_config1(ctx) if rank == 0 and args.workload == WORKLOAD and not args.no_e2e
               else None)

    # e2e through the drop-in call with host buffers
    e2e = None
    if not args.no_e2e:
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        e2e = e2e_arm(args, ctx, graphs, setup, per_step)
        if world > 1:
            # whole job: every rank's chain-steps over the slowest rank's time
            import torch.distributed as dist
            el = torch.tensor([e2e["elapsed_s"]], dtype=torch.float64, device="cuda")
            dist.all_reduce(el, op=dist.ReduceOp.MAX)
            e2e["value"] = e2e["chain_steps"] * world / float(el.item())
    plain = None
    if not args.no_plain:
        plain = plain_kernel_arm(graphs, setup, args.plain_sweeps, ctx)
    if plain and "value" in plain:
        # identical trajectories: the plain kernel needs the same sweeps; its
        # time follows from its measured chain-steps/s on this workload
        for e in tt:
            e["plain_seconds_est"] = e["sweeps"] * len(graphs) * args.chains / plain["value"]
    batched = None if args.no_batched else batched_arm(args, ctx)
    ingest = ingest_arm(args, ctx, graphs, setup) if args.ingest else None
    serving = None
    serving_mixed = None
    if not args.no_serving:
        rates = [float(x) for x in str(args.serve_rate).split(",") if x]
        runs = [serving_arm(args, ctx, r, compare_offline=(r == rates[-1])) for r in rates]
        serving = runs[0] if len(runs) == 1 else runs
        budgets = [int(float(x)) for x in str(args.serve_budgets).split(",") if x]
        if budgets and args.serve_mixed_rate > 0:
            serving_mixed = serving_arm(args, ctx, args.serve_mixed_rate, budgets=budgets,
                                        max_requests=args.serve_mixed_requests)

    peaks = measured_peaks()
    sm_count = ctx.info()["sm_count"]
    sm_mhz = clk["sm_mhz"] or peaks.get("sm_max_mhz", 2070.0)
    smem_peak = sm_count * 128.0 * sm_mhz * 1e6 / 1e9   # GB/s
    achieved = sum(step_bytes) / (total_ms / 1e3) / 1e9
    # The committed profile figures (DRAM bytes and instructions per
    # chain-sweep) describe the headline workload's kernel only.
    traffic = profile_traffic() if args.workload == WORKLOAD else None
    result = {
        "metric": "chain-steps/s",
        "value": value,
        "unit": "chain-steps/s",
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": total_ms / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": ("synthetic (seeded torus 50x60 +-1 and Erdos-Renyi n=2000 d~19 +-1)"
                 if args.workload == WORKLOAD else
                 "synthetic (seeded torus 100x200 +-1, random tree n=10000 +1, Erdos-Renyi n=5000 d~5 +-1)"),
        "config": {
            "workload": args.workload,
            "graphs": [dict(name=g.name, n=g.n, m=g.m, B=g.max_weighted_degree()) for g in graphs],
            "chains_per_graph": args.chains,
            "sweeps_per_chain": sweeps,
            "sweeps_per_step": per_step,
            "phases": phases,
            "t0_ladder": LADDER,
            "threads_per_chain": info["threads_per_chain"],
            "chains_per_cta": info["chains_per_cta"],
            "grid": info["grid"],
            "csr": {1: "unit16 in shared memory", 2: "packed32 in shared memory",
                    3: "HBM, 8-byte entries", 4: "HBM, 16-bit entries",
                    5: "HBM, 32-bit entries"}[info["csr_format"]],
            "gain_bytes": info["gain_width"],
            "items": info["items"],
            "balanced_items": bool(info["balanced"]),
            "score_path": "int64" if info["score64"] else "int32",
            "launch_classes": info.get("launch_classes"),
            "plan": "rfmf_autotune (measured)" if tuned else "planner rules",
            "autotune": tuned,
            "l2": "flushed (256 MB write) between timed steps",
            "parallelism": f"replicas x{world}",
        },
        # kernel launches of the timed steps, counted by the library (a step
        # of a multi-graph class is cut at phase boundaries)
        "gpu_launches": timed_launches,
        "e2e": e2e,
        "config1_gpu": config1,
        "time_to_target": tt,
        "serving": serving,
        "serving_mixed_budgets": serving_mixed,
        "ingest_output": ingest,
        "clocks": clk,
        "roofline": {
            "bound": "smem",
            "achieved": achieved,
            "peak": smem_peak,
            "unit": "GB/s",
            "frac": achieved / smem_peak,
            "traffic": (traffic or {}).get("dram_bytes_per_launch"),
            "traffic_note": ("DRAM bytes per launch from profiles/anneal_kernel_traffic.json "
                             "(ncu, same kernel shape, %s-sweep windows); the working set is "
                             "shared-memory/L2 resident" % (traffic or {}).get("window_sweeps")),
            "peak_source": f"{sm_count} SMs x 128 B/clk x {sm_mhz:.0f} MHz (median SM clock sampled "
                           "during the timed region)",
            "bytes_model": "5n + min(P,n)(8 + 16 dbar) per chain-sweep + n per improving sweep",
        },
        "issue_roofline": issue_roofline(traffic, value, sm_count, sm_mhz),
        "wall_s": wall,
        "step_ms": [round(m, 3) for m in step_ms],
        # the >= 5x comparisons last: the plain one-graph-per-launch kernel
        # (the reference's own) against the batched form on identical samples
        "plain_kernel": plain,
        "batched": batched,
    }
    return result


def issue_roofline(traffic, value, sm_count, sm_mhz):
    """The bound this integer kernel actually meets: warp instructions per
    chain-sweep (ncu, same kernel and workload, from the profile summary)
    times chain-steps/s, against 4 issue slots per SM per cycle."""
    ipc = (traffic or {}).get("warp_inst_per_chain_sweep")
    if not ipc:
        return None
    achieved = value * ipc / 1e12
    peak = sm_count * 4.0 * sm_mhz * 1e6 / 1e12
    return {"bound": "integer issue", "achieved": achieved, "peak": peak, "unit": "T warp-inst/s",
            "frac": achieved / peak, "warp_inst_per_chain_sweep": ipc,
            "source": "profiles/anneal_kernel_traffic.json (ncu smsp__inst_executed.sum / chain-sweeps)",
            "peak_source": f"{sm_count} SMs x 4 warp-inst/clk x {sm_mhz:.0f} MHz"}


def plain_kernel_arm(graphs, setup, sweeps, ctx):
    """The reference's own kernel (one graph per launch, one block per chain,
    state in global memory), compiled from its sources for sm_103a and
    launched through oracle/refgpu.py, on a bounded sample of the same
    workload; against librfmf.so on the identical sample in two forms: the
    batched form (both graphs' chains in one batch, one launch per phase)
    and the annealGpu drop-in (one rfmf_anneal call per graph).  All three
    must give identical results chain for chain."""
    sys.path.insert(0, str(ROOT / "oracle"))
    try:
        import refgpu
    except Exception as e:   # pragma: no cover
        return {"unavailable": f"harness import failed: {e}"}
    if not refgpu.available():
        return {"unavailable": "reference kernel cubin (oracle/_ref) not built on this machine"}
    import torch

    import rfmf_gb300 as R
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    phases, iters = schedule(sweeps)
    ref_ms = ours_ms = 0.0
    cs = 0
    tpbs = []
    refs = []
    dgs = [R.DeviceGraph(ctx, s["g"]) for s in setup]
    for s, dg in zip(setup, dgs):
        g = s["g"]
        r = refgpu.run(g, s["init"], s["t0s"], s["solver"], phases, iters, sms)
        refs.append(r)
        ref_ms += r["ms"]
        tpbs.append(r["tpb"])
        o = R.anneal_gpu(ctx, dg, g.max_weighted_degree(), s["init"], s["t0s"], phases, iters,
                         s["solver"])
        ours_ms += o.kernel_ms
        cs += len(s["seeds"]) * sweeps
        same = (np.array_equal(o.best_spins, r["best_spins"]) and
                np.array_equal(o.end_spins, r["end_spins"]) and
                np.array_equal(o.best_vals, r["best_vals"]))
        if not same:
            raise AssertionError(f"reference kernel and librfmf.so differ on {g.name}")
    gl, ini, sol, t0 = [], [], [], []
    for s, dg in zip(setup, dgs):
        gl += [dg] * len(s["seeds"])
        ini += list(s["init"])
        sol += s["solver"]
        t0 += s["t0s"]
    b = R.Batch(ctx, gl, t0, sol, ini, phases, iters)
    batch_ms = b.run_timed(sweeps)
    out = b.read()
    b.close()
    for d in dgs:
        d.close()
    c0 = 0
    for s, r in zip(setup, refs):
        C = len(s["seeds"])
        if not (np.array_equal(np.stack(out["best_spins"][c0:c0 + C]), r["best_spins"]) and
                np.array_equal(np.stack(out["end_spins"][c0:c0 + C]), r["end_spins"]) and
                np.array_equal(out["best_vals"][c0:c0 + C], r["best_vals"])):
            raise AssertionError(f"reference kernel and the batched form differ on {s['g'].name}")
        c0 += C
    plain = cs / (ref_ms / 1e3)
    batched = cs / (batch_ms / 1e3)
    dropin = cs / (ours_ms / 1e3)
    return {"value": plain, "unit": "chain-steps/s",
            "ours_batched": batched, "ours_dropin": dropin,
            "speedup_vs_plain": batched / plain, "dropin_speedup_vs_plain": dropin / plain,
            "sample": f"{len(setup)} graphs x {len(setup[0]['seeds'])} chains x {sweeps} sweeps "
                      f"(phases 128..1); reference threads/block {tpbs}",
            "identical_results": True,
            "what": "reference mcKernel (its sources built for sm_103a), one launch per graph, "
                    "kernel-only cudaEvent time; ours: both graphs in one batch (one launch per phase), and "
                    "rfmf_anneal per graph"}


def _median_time(fn, reps=3):
    fn()
    ts = []
    for _ in range(reps):
        t = time.perf_counter()
        out = fn()
        ts.append(time.perf_counter() - t)
    return statistics.median(ts), out


def ingest_arm(args, ctx, graphs, setup):
    """Graph ingest and output path, each against its host equivalent.

    Ingest: rfmf_graph_from_edges (edge list in host memory -> CSR built on the
    device: dense ids, degree count, scatter, row sort, dedupe, compact
    formats) against graphs.csr_from_edges (numpy, one core) on the large
    sparse shapes plus an Erdos-Renyi n = 20000 mean degree 48 graph, edges
    in shuffled order; the two CSRs must be equal.  Output: rfmf_batch_cuts
    (every chain's cut recomputed on the device) and rfmf_batch_partitions
    (the '0'/'1' partition strings) for the 2048 chains of the bench workload
    after 1000 sweeps, against rfmf_cut_value per chain and numpy strings on
    the host; the results must be equal.  Wall times (median of 3 after one
    warm-up call) of the public calls, host<->device copies included."""
    import rfmf_gb300 as R
    rng = np.random.default_rng(23)
    ing = []
    for g in (R.torus(100, 200, signed=True, seed=0, name="torus100x200"),
              R.random_tree(10000, seed=0, name="tree10000"),
              R.erdos_renyi_sparse(5000, 5, signed=True, seed=0, name="er5000_d5"),
              R.erdos_renyi_degree(20000, 48, signed=True, seed=0, name="er20000_d48")):
        rows = np.repeat(np.arange(g.n), np.diff(g.offsets.astype(np.int64)))
        up = g.col > rows
        u, v, w = rows[up], g.col[up].astype(np.int64), g.weight[up].astype(np.int64)
        perm = rng.permutation(len(u))
        u, v, w = u[perm], v[perm], w[perm]
        t_dev, dg = _median_time(lambda: R.DeviceGraph.from_edges(ctx, u, v, w))
        t_host, hg = _median_time(lambda: R.csr_from_edges(u, v, w))
        off, col, wt = dg.csr()
        same = (np.array_equal(off, hg.offsets) and np.array_equal(col, hg.col) and
                np.array_equal(wt, hg.weight))
        dg.close()
        if not same:
            raise AssertionError(f"device CSR of {g.name} differs from the host build")
        ing.append({"graph": g.name, "n": g.n, "edges": int(len(u)), "device_ms": t_dev * 1e3,
                    "host_numpy_ms": t_host * 1e3, "device_edges_per_s": len(u) / t_dev,
                    "speedup": t_host / t_dev})

    dgs = [R.DeviceGraph(ctx, s["g"]) for s in setup]
    gl, ini, sol, t0 = [], [], [], []
    for k, s in enumerate(setup):
        gl += [dgs[k]] * len(s["seeds"])
        ini += list(s["init"])
        sol += s["solver"]
        t0 += s["t0s"]
    b = R.Batch(ctx, gl, t0, sol, ini, list(PHASES), [125] * len(PHASES))
    b.run(1000)
    out = b.read()
    C = len(ini)
    t_cut_dev, cuts = _median_time(lambda: b.cuts(best=False))
    t_par_dev, parts = _median_time(lambda: b.partitions(best=False))
    owners = [s["g"] for s in setup for _ in s["seeds"]]
    t_cut_host, hcuts = _median_time(
        lambda: np.array([R.cut_value(g, sp) for g, sp in zip(owners, out["end_spins"])]))
    t_par_host, hparts = _median_time(
        lambda: [np.where(sp > 0, ord("1"), ord("0")).astype(np.uint8).tobytes().decode()
                 for sp in out["end_spins"]])
    if not (np.array_equal(cuts, hcuts) and parts == hparts):
        raise AssertionError("device output path differs from the host recompute")
    b.close()
    for d in dgs:
        d.close()
    nsum = sum(len(p) for p in parts)
    return {"ingest": ing,
            "output": {"chains": C, "vertices_total": nsum,
                       "cuts_device_ms": t_cut_dev * 1e3, "cuts_host_ms": t_cut_host * 1e3,
                       "partitions_device_ms": t_par_dev * 1e3,
                       "partitions_host_ms": t_par_host * 1e3},
            "what": "wall time of the public calls (median of 3 after a warm-up), host<->device "
                    "copies included; host: numpy CSR build, rfmf_cut_value per chain, numpy "
                    "strings; results equal"}


def batched_graphs(count, seed=0):
    """Uneven graphs for the batched form: sizes log-uniform in [800, 20000],
    families 1/3 each (Erdos-Renyi with mean degree 5-48, toroidal grid,
    random planar-like with mean degree ~11.7), weights +-1 or +1 alternating."""
    import math

    import rfmf_gb300 as R
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(round(math.exp(rng.uniform(math.log(800), math.log(20000)))))
        signed = bool(i % 2)
        fam = i % 3
        if fam == 0:
            g = R.erdos_renyi_sparse(n, float(rng.uniform(5, 48)), signed=signed, seed=1000 + i,
                                     name=f"er{n}")
        elif fam == 1:
            rows = max(3, int(math.sqrt(n)))
            g = R.torus(rows, max(3, n // rows), signed=signed, seed=1000 + i,
                        name=f"torus{rows}x{max(3, n // rows)}")
        else:
            g = R.planar_like(n, 11.7, signed=signed, seed=1000 + i, name=f"planar{n}")
        out.append(g)
    return out


def _timed_graph_windows(ctx, batch, sweeps, window):
    """Advance `batch` by `sweeps` sweeps as CUDA-graph replays of fixed
    `window`-sweep launches (captured once before the clock), timed with
    CUDA events on the library's stream."""
    import torch
    launches = max(1, sweeps // window)
    assert launches * window == sweeps, "sweeps must be a multiple of the window"
    batch.run_graph(window, launches, 0)          # capture + instantiate only
    st = torch.cuda.ExternalStream(ctx.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    batch.run_graph(window, launches, 1)
    e1.record(st)
    batch.synchronize()
    return e0.elapsed_time(e1), launches


def batched_arm(args, ctx):
    """The batched form: G uneven graphs x 64 chains, all in one batch whose
    sweeps run as CUDA-graph replays of fixed-size windows (work queue over
    graphs, launch classes and chains per CTA from the planner).  Against the
    plain kernel: the reference's kernel launched once per graph, as it runs,
    on the first args.batched_plain_graphs graphs, with our batched form on
    that same subset; both advance every chain the same sweeps and the
    results must be identical chain for chain."""
    import torch

    import rfmf_gb300 as R
    sys.path.insert(0, str(ROOT / "oracle"))
    t = time.perf_counter()
    graphs = batched_graphs(args.batched_graphs)
    gen_s = time.perf_counter() - t
    C = 64
    sweeps = args.batched_sweeps
    window = args.batched_window
    phases, iters = schedule(sweeps)
    dgs = [R.DeviceGraph(ctx, g) for g in graphs]
    setup = []
    for i, g in enumerate(graphs):
        seeds = [5_000_000 + C * i + k for k in range(C)]
        setup.append(dict(init=np.stack([R.initial_spins(x, g.n) for x in seeds]),
                          solver=[R.solver_seed(x) for x in seeds],
                          t0s=[LADDER[k % 8] for k in range(C)]))

    def make_batch(idx):
        gl, ini, sol, t0 = [], [], [], []
        for i in idx:
            gl += [dgs[i]] * C
            ini += list(setup[i]["init"])
            sol += setup[i]["solver"]
            t0 += setup[i]["t0s"]
        return R.Batch(ctx, gl, t0, sol, ini, phases, iters)

    every = list(range(len(graphs)))
    # warm-up batch (learned per-graph costs feed the work-item sizing)
    wb = make_batch(every)
    wb.run_timed(min(sweeps, 2000))
    wb.close()
    b = make_batch(every)
    ms, launches = _timed_graph_windows(ctx, b, sweeps, window)
    info = b.info()
    done = b.read()["sweeps_done"]
    b.close()
    if not all(int(d) == sweeps for d in done):
        raise AssertionError("batched form: not every chain finished its schedule")
    chain_steps = len(graphs) * C * sweeps
    res = {"value": chain_steps / (ms / 1e3), "unit": "chain-steps/s", "graphs": len(graphs),
           "chains_per_graph": C, "sweeps": sweeps, "window_sweeps": window,
           "launch_windows": launches, "launches_per_window": info["launch_classes"],
           "form": "CUDA-graph replay of fixed-size sweep windows", "kernel_ms": ms,
           "plan": {k: info[k] for k in ("threads_per_chain", "chains_per_cta", "grid", "items",
                                         "csr_format", "gain_width", "balanced",
                                         "launch_classes")},
           "n_range": [min(g.n for g in graphs), max(g.n for g in graphs)],
           "graph_gen_s": gen_s}
    try:
        import refgpu
    except Exception as e:   # pragma: no cover
        res["plain_kernel"] = {"unavailable": f"harness import failed: {e}"}
        return res
    if not refgpu.available():
        res["plain_kernel"] = {"unavailable": "reference kernel cubin (oracle/_ref) not built"}
        return res
    sub = every[:min(args.batched_plain_graphs, len(graphs))]
    b = make_batch(sub)
    ms_sub, _ = _timed_graph_windows(ctx, b, sweeps, window)
    out = b.read()
    b.close()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    ref_ms = 0.0
    same = True
    for k, i in enumerate(sub):
        st = setup[i]
        r = refgpu.run(graphs[i], st["init"], st["t0s"], st["solver"], phases, iters, sms)
        ref_ms += r["ms"]
        sl = slice(k * C, (k + 1) * C)
        same = same and np.array_equal(np.stack(out["best_spins"][sl]), r["best_spins"]) and \
            np.array_equal(np.stack(out["end_spins"][sl]), r["end_spins"]) and \
            np.array_equal(out["best_vals"][sl], r["best_vals"])
    for d in dgs:
        d.close()
    if not same:
        raise AssertionError("batched results differ from the reference kernel")
    cs_sub = len(sub) * C * sweeps
    plain = cs_sub / (ref_ms / 1e3)
    ours = cs_sub / (ms_sub / 1e3)
    res["plain_kernel"] = {"value": plain, "unit": "chain-steps/s", "graphs": len(sub),
                           "launches": len(sub), "kernel_ms": ref_ms, "ours_same_graphs": ours,
                           "ours_kernel_ms": ms_sub, "identical_results": bool(same),
                           "what": "reference mcKernel (sm_103a build of its sources), one "
                                   "launch per graph, kernel-only cudaEvent time, on the first "
                                   f"{len(sub)} graphs; ours on the same graphs in one batch"}
    res["speedup_vs_plain"] = ours / plain
    return res


def serving_graphs():
    import rfmf_gb300 as R
    out = []
    for k, n in enumerate((5000, 10000, 20000)):
        rows = int(n ** 0.5)
        out.append(R.torus(rows, n // rows, signed=True, seed=k, name=f"torus{rows}x{n // rows}"))
        out.append(R.random_tree(n, seed=k, name=f"tree{n}"))
        out.append(R.erdos_renyi_sparse(n, 5, signed=True, seed=k, name=f"er{n}_d5"))
    return out


def serving_arm(args, ctx, rate, budgets=None, max_requests=None, compare_offline=False):
    """Continuous batching through the request server: Poisson arrivals at
    `rate` req/s for `seconds`, or until max_requests (default
    args.serve_max_requests) have arrived (which bounds the high-rate runs:
    at 2000 req/s the cap's requests arrive in a fraction of a second and the
    run measures the saturated server); each request draws a graph from the
    large-sparse families (torus, tree, ER d=5; n 5000-20000), 16-256 chains
    and a sweep budget (default schedule): args.serve_sweeps, or drawn
    uniformly from `budgets` when given, so that short and long requests
    share windows.  Latency = submit -> results on the host (server clock).
    `offered_rate_req_s` is the rate at which the submitting thread actually
    handed requests to the server."""
    import threading

    import rfmf_gb300 as R
    graphs = serving_graphs()
    dgs = [R.DeviceGraph(ctx, g) for g in graphs]
    rng = np.random.default_rng(17)
    seconds = args.serve_seconds
    arrivals = []
    t = 0.0
    cap = max_requests or args.serve_max_requests
    while len(arrivals) < cap:
        t += float(rng.exponential(1.0 / rate))
        if t > seconds:
            break
        arrivals.append(t)
    submitted = [0.0] * len(arrivals)
    reqs = [dict(g=int(rng.integers(len(graphs))), C=int(rng.choice([16, 32, 64, 128, 256])),
                 seed0=10_000_000 + 1000 * i,
                 sweeps=int(rng.choice(budgets)) if budgets else args.serve_sweeps)
            for i in range(len(arrivals))]
    srv = R.Server(ctx, window_sweeps=args.serve_window)
    ids = [None] * len(reqs)
    err = []
    submit_s = []     # duration of each Server.submit call (rfmf_submit + Python marshalling)

    # Request inputs are built before the arrival stream starts, so that the
    # submitting thread only calls submit (building initial spins in the loop
    # had capped the offered rate near 180 req/s).
    inputs = []
    for r in reqs:
        g = graphs[r["g"]]
        seeds = [r["seed0"] + k for k in range(r["C"])]
        inputs.append((np.stack([R.initial_spins(x, g.n) for x in seeds]),
                       [LADDER[k % 8] for k in range(r["C"])],
                       [R.solver_seed(x) for x in seeds]))

    def submitter():
        t0 = time.perf_counter()
        for i, (at, r) in enumerate(zip(arrivals, reqs)):
            init, t0s, solver = inputs[i]
            d = at - (time.perf_counter() - t0)
            if d > 0:
                time.sleep(d)
            try:
                phases, iters = schedule(r["sweeps"])
                ts = time.perf_counter()
                ids[i] = srv.submit(dgs[r["g"]], init, t0s, phases, iters, solver)
                submit_s.append(time.perf_counter() - ts)
                submitted[i] = time.perf_counter() - t0
            except Exception as e:   # pragma: no cover
                err.append(repr(e))
                return

    th = threading.Thread(target=submitter)
    t_start = time.perf_counter()
    th.start()
    th.join()
    if err:
        raise RuntimeError(err[0])
    lat, cs = [], 0
    lat_by_budget = {}
    for i, r in enumerate(reqs):
        st = srv.wait(ids[i], timeout=600)
        if st["state"] != "done":
            raise RuntimeError(f"request {i} {st['state']}")
        lat.append(st["finish_s"] - st["submit_s"])
        lat_by_budget.setdefault(r["sweeps"], []).append(lat[-1])
        res = srv.result(ids[i])
        g = graphs[r["g"]]
        if res.best_vals[0] != g.cut_value(res.best_spins[0]):
            raise AssertionError("served best cut disagrees with its spins")
        cs += r["C"] * r["sweeps"]
    wall = time.perf_counter() - t_start
    stats = srv.stats()
    srv.close()
    # The same requests' chains as ONE offline batch (one schedule: only when
    # every request has the same budget): what continuous batching costs
    # against knowing the whole workload up front.
    offline = None
    if compare_offline and not budgets and args.serve_offline:
        gl, ini, sol, t0 = [], [], [], []
        for i, r in enumerate(reqs):
            init, t0s, solver = inputs[i]
            gl += [dgs[r["g"]]] * r["C"]
            ini += list(init)
            sol += solver
            t0 += t0s
        phases, iters = schedule(args.serve_sweeps)
        b = R.Batch(ctx, gl, t0, sol, ini, phases, iters)
        ms = b.run_timed(args.serve_sweeps)
        b.close()
        offline = {"chain_steps_per_s": len(ini) * args.serve_sweeps / (ms / 1e3), "kernel_ms": ms,
                   "what": "every request's chains in one batch, one launch (device time)"}
    lat = np.array(lat)
    span = submitted[-1] - submitted[0] if len(submitted) > 1 else 0.0
    return {"rate_req_s": rate, "requests": len(reqs),
            "arrival_window_s": arrivals[-1] if arrivals else 0.0,
            "offered_rate_req_s": (len(submitted) - 1) / span if span > 0 else None,
            "submit_ms_p50": float(np.percentile(submit_s, 50) * 1e3) if submit_s else None,
            "submit_ms_p99": float(np.percentile(submit_s, 99) * 1e3) if submit_s else None,
            "sweeps_per_request": sorted(set(r["sweeps"] for r in reqs)),
            "window_sweeps": args.serve_window,
            "latency_by_budget": {str(k): {"requests": len(v), "p50_s": float(np.percentile(v, 50)),
                                           "p99_s": float(np.percentile(v, 99))}
                                  for k, v in sorted(lat_by_budget.items())},
            "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p99_s": float(np.percentile(lat, 99)),
            "latency_max_s": float(lat.max()),
            "chain_steps_per_s": cs / wall, "wall_s": wall,
            "gpu_busy_frac": stats["kernel_s"] / wall, "windows": stats["windows"],
            "kernel_chain_steps_per_s": stats["chain_sweeps"] / max(stats["kernel_s"], 1e-9),
            "offline_batch_same_requests": offline,
            "launches": stats["launches"],
            "mix": "graphs torus/tree/ER-d5 at n 5000/10000/20000; chains 16-256 uniform over "
                   "{16,32,64,128,256}; Poisson arrivals"}


def e2e_arm(args, ctx, graphs, setup, per_step):
    """End to end through the drop-in: per step and graph, rfmf_graph_create
    (host CSR -> device) and one rfmf_anneal call (host spins in, host spins
    and cuts out), all inside the clock.  The breakdown splits the wall time
    into graph upload, the annealing kernel's own device time, and the rest of
    each rfmf_anneal call (beta tables, batch set-up and copies, read-back)."""
    import rfmf_gb300 as R
    phases, iters = schedule(per_step)
    K = min(args.steps, 2)
    # Each call's plan measured once per shape, before the clock (a caller
    # issuing many calls of one shape tunes once; the pick is cached in the
    # context and passed as the call's launch config).
    cfgs = []
    for s in setup:
        if args.no_autotune:
            cfgs.append(R.make_config())
            continue
        dg = R.DeviceGraph(ctx, s["g"])
        cfg, _ = R.autotune(ctx, [dg] * len(s["seeds"]), s["t0s"], s["solver"], list(s["init"]),
                            phases, iters)
        cfgs.append(cfg)
        dg.close()
    h2d = d2h = 0
    t_graph = t_call = kern = 0.0
    t = time.perf_counter()
    for _ in range(K):
        for s, cfg in zip(setup, cfgs):
            g = s["g"]
            t1 = time.perf_counter()
            dg = R.DeviceGraph(ctx, g)
            t2 = time.perf_counter()
            res = R.anneal_gpu(ctx, dg, g.max_weighted_degree(), s["init"], s["t0s"], phases,
                               iters, s["solver"], cfg)
            t3 = time.perf_counter()
            dg.close()
            t_graph += t2 - t1
            t_call += t3 - t2
            kern += res.kernel_ms / 1e3
            C = len(s["seeds"])
            words = (g.n + 31) // 32
            runs = len(R.beta_tables(sorted(set(s["t0s"])), per_step)[0])
            h2d += ((g.n + 1) * 4 + 2 * g.m * 8 + 2 * C * words * 4 + C * (96 + 4) + runs * 12 +
                    len(phases) * 12)
            d2h += 2 * C * words * 4 + C * 96
            assert res.best_vals[0] == g.cut_value(res.best_spins[0])
    el = time.perf_counter() - t
    chain_steps = K * sum(len(s["seeds"]) for s in setup) * per_step
    return {"value": chain_steps / el, "unit": "chain-steps/s", "elapsed_s": el,
            "chain_steps": chain_steps,
            "h2d_bytes_per_step": h2d // K, "d2h_bytes_per_step": d2h // K,
            "breakdown_s": {"graph_upload": t_graph, "anneal_kernel": kern,
                            "anneal_call_other": t_call - kern,
                            "outside_calls": el - t_graph - t_call},
            "kernel_only_rate": chain_steps / kern,
            "plans": [{"threads_per_chain": c.threads_per_chain, "csr_format": c.csr_format}
                      for c in cfgs],
            "api": "rfmf_graph_create + rfmf_anneal (annealGpu drop-in), host buffers, one call "
                   f"per graph, {per_step} sweeps per chain per call"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sweeps", type=int, default=10_000_000)
    ap.add_argument("--phases", default=None,
                    help="comma list of P for the main workload (default 128,...,1; profiling cases "
                         "use one phase)")
    ap.add_argument("--chains", type=int, default=None, help="chains per graph (default per workload)")
    ap.add_argument("--workload", default=WORKLOAD, choices=[WORKLOAD, LARGE_WORKLOAD],
                    help="the headline mid-size workload (default) or the large sparse shapes, "
                         "a profiling case (no e2e, CPU or plain-kernel legs)")
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--chains-per-cta", type=int, default=0)
    ap.add_argument("--csr-format", type=int, default=0,
                    help="0 auto; 1/2 shared-memory 16/32-bit entries; 3 HBM compact entries; "
                         "4 HBM 8-byte entries (profiling cases)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="plan the batch with the planner's rules instead of measuring candidates")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--plain-sweeps", type=int, default=16000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-graphs", type=int, default=512)
    ap.add_argument("--batched-sweeps", type=int, default=20000)
    ap.add_argument("--batched-window", type=int, default=2500,
                    help="sweeps per CUDA-graph window of the batched form")
    ap.add_argument("--batched-plain-graphs", type=int, default=128,
                    help="graphs of the batched mix also run on the plain kernel")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--ingest", action="store_true",
                    help="also time graph ingest and the output path against their host equivalents")
    ap.add_argument("--serve-rate", default="2,10,100,2000",
                    help="req/s; a comma list sweeps several rates")
    ap.add_argument("--serve-seconds", type=float, default=20.0,
                    help="longest arrival window per rate")
    ap.add_argument("--serve-max-requests", type=int, default=200,
                    help="arrivals per rate at most (bounds the high-rate runs)")
    ap.add_argument("--serve-sweeps", type=int, default=100_000)
    ap.add_argument("--serve-window", type=int, default=4096)
    ap.add_argument("--serve-budgets", default="100000,1000000",
                    help="sweep budgets mixed in one serving run (10^7 adds minutes of wall time)")
    ap.add_argument("--serve-mixed-rate", type=float, default=10.0,
                    help="req/s of the mixed-budget serving run (0 = skip)")
    ap.add_argument("--serve-mixed-requests", type=int, default=40)
    ap.add_argument("--serve-offline", type=int, default=1,
                    help="also run each fixed-budget serving mix as one offline batch (1) or not (0)")
    args = ap.parse_args()
    if args.chains is None:
        args.chains = WORKLOAD_CHAINS[args.workload]
    if args.workload != WORKLOAD:
        args.no_e2e = args.no_cpu = args.no_plain = True

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        graphs = workload_graphs()
        per_step_s = max(2.0, 60.0 / max(args.steps + args.warmup, 1))
        rate, cores, sample, el = cpu_rate(graphs, args.steps, args.warmup, per_step_s)
        line = {
            "impl": "reference", "metric": "chain-steps/s", "value": rate,
            "unit": "chain-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int64", "data": "synthetic", "config": {"workload": WORKLOAD},
            "cpu_baseline": {"value": rate, "unit": "chain-steps/s", "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": "chain-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference ships no CPU annealer; this is the oracle's C restatement "
                    "of its sweep (src/anneal_kernels.cu:262-491), one chain per core",
        }
        print(json.dumps(line))
        return 0

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    res = gpu_arm(args, rank, world)
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, cores, sample, _ = cpu_rate(workload_graphs(), 1, 0, args.cpu_seconds)
        res["cpu_baseline"] = {"value": rate, "unit": "chain-steps/s", "cores": cores,
                               "kind": "port", "sample": sample}
        res["cpu_config1"] = cpu_config1(min(6.0, args.cpu_seconds))
    # keep the plain-kernel comparisons at the end of the line, with a short
    # summary after them
    for k in ("plain_kernel", "batched"):
        res[k] = res.pop(k, None)
    pk, bt = res.get("plain_kernel") or {}, res.get("batched") or {}
    res["vs_plain_kernel"] = {
        "batched_same_sample": pk.get("speedup_vs_plain"),
        "dropin_same_sample": pk.get("dropin_speedup_vs_plain"),
        "batched_512_graph_mix": bt.get("speedup_vs_plain"),
        "identical_results": bool(pk.get("identical_results") and
                                  (bt.get("plain_kernel") or {}).get("identical_results")),
    }
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
