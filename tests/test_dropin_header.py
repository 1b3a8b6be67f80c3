"""The C++ drop-in (include/rfmf_annealgpu.hpp, gpu3::annealGpu with the
reference's signature, src/anneal_gpu.cuh:76-88) compiled into a C++ caller
of its own (tests/dropin/annealgpu_caller.cpp, which restates the
reference's interface types) and run as a separate process against
librfmf.so: on a GPU its outputs equal the oracle's chain for chain (end and
best spins, final and best cut values; integer work, zero tolerance) and
*kernelMs is filled; everywhere, a mismatched argument list exits non-zero
with the reference's message (src/anneal_kernels.cu:848-855) before any
device call.  The reference's own main.cu linked against the same header is
covered where its sources exist (test_dropin_link.py)."""
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, chains_for


@pytest.fixture(scope="module")
def caller(rfmf, tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    rfmf.lib()
    libdir = ROOT / "rfmf_gb300" / "_build"
    exe = tmp_path_factory.mktemp("dropin") / "annealgpu_caller"
    r = subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}",
                        str(ROOT / "tests" / "dropin" / "annealgpu_caller.cpp"),
                        f"-L{libdir}", "-lrfmf", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def _write_input(path, g, init, t0s, solver, phases, iters, B):
    C, n = init.shape
    with open(path, "wb") as f:
        np.array([n, len(g.col), C, len(phases), B], np.int64).tofile(f)
        g.offsets.astype(np.uint32).tofile(f)
        g.col.astype(np.int32).tofile(f)
        g.weight.astype(np.int32).tofile(f)
        init.astype(np.int8).tofile(f)
        np.array(t0s, np.float64).tofile(f)
        np.array(solver, np.uint64).tofile(f)
        np.array(phases, np.uint64).tofile(f)
        np.array(iters, np.uint64).tofile(f)


def _case(rfmf):
    g = rfmf.erdos_renyi(400, 0.025, signed=True, seed=11)
    seeds = list(range(40, 52))
    init, solver = chains_for(g, seeds)
    t0s = [35.0, 50.0, 70.0, 100.0, 140.0, 200.0] * 2
    return g, init, solver, t0s, [16, 4, 1], [150, 150, 150]


def test_argument_check_exits_before_device_work(rfmf, caller, tmp_path):
    g, init, solver, t0s, phases, iters = _case(rfmf)
    _write_input(tmp_path / "in.bin", g, init, t0s, solver, phases, iters,
                 g.max_weighted_degree())
    r = subprocess.run([str(caller), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), "drop"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode != 0
    assert "annealGpu needs non-empty, equal-length t0s (12), solverSeeds (11)" in r.stderr
    assert not (tmp_path / "out.bin").exists()


@pytest.mark.gpu
def test_annealgpu_header_matches_oracle(rfmf, oracle, caller, tmp_path):
    g, init, solver, t0s, phases, iters = _case(rfmf)
    C, n = init.shape
    B = g.max_weighted_degree()
    _write_input(tmp_path / "in.bin", g, init, t0s, solver, phases, iters, B)
    r = subprocess.run([str(caller), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    raw = (tmp_path / "out.bin").read_bytes()
    end = np.frombuffer(raw, np.int8, C * n, 0).reshape(C, n)
    best = np.frombuffer(raw, np.int8, C * n, C * n).reshape(C, n)
    vals = np.frombuffer(raw, np.int64, 2 * C, 2 * C * n)
    ms = np.frombuffer(raw, np.float32, 1, 2 * C * n + 16 * C)[0]
    ref = oracle.anneal(g, init, t0s, solver, phases, iters)
    assert np.array_equal(end, ref["end_spins"])
    assert np.array_equal(best, ref["best_spins"])
    assert np.array_equal(vals[:C], ref["best_vals"])
    assert np.array_equal(vals[C:], ref["cur_vals"])
    assert ms > 0
    assert f"chains {C}" in r.stdout
