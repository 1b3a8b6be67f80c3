"""ctypes bindings for the oracle library (oracle/_build/librfmf_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the oracle.  The product never imports it.
"""
import ctypes as ct
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "librfmf_oracle.so"

_P = ct.c_void_p
_I64 = ct.c_int64
_U64 = ct.c_uint64

_lib = None


def build(quiet=True):
    """Compile the oracle with make (plain C, a few seconds)."""
    out = subprocess.run(["make", "-C", str(HERE), "-s"], capture_output=quiet, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{out.stdout}\n{out.stderr}")
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ct.CDLL(str(LIB_PATH))
        L.rfmf_oracle_philox_block.argtypes = [_U64, _U64, _U64, _P]
        L.rfmf_oracle_philox_block.restype = None
        L.rfmf_oracle_gumbel.argtypes = [ct.c_uint32]
        L.rfmf_oracle_gumbel.restype = ct.c_int32
        L.rfmf_oracle_beta_fixed.argtypes = [_U64, ct.c_double]
        L.rfmf_oracle_beta_fixed.restype = ct.c_int32
        L.rfmf_oracle_score_safe_int32.argtypes = [_I64, ct.c_double, _I64]
        L.rfmf_oracle_score_safe_int32.restype = ct.c_int
        L.rfmf_oracle_max_weighted_degree.argtypes = [_I64, _P, _P]
        L.rfmf_oracle_max_weighted_degree.restype = _I64
        L.rfmf_oracle_cut_value.argtypes = [_I64, _P, _P, _P, _P]
        L.rfmf_oracle_cut_value.restype = _I64
        L.rfmf_oracle_initial_spins.argtypes = [_U64, _I64, _P]
        L.rfmf_oracle_initial_spins.restype = None
        L.rfmf_oracle_anneal_window.argtypes = [
            _I64, _P, _P, _P, _I64, _P, _P, _I64, _P, _P, _U64, _U64,
            _P, _P, _P, _P, _P, ct.c_int]
        L.rfmf_oracle_anneal_window.restype = ct.c_int
        L.rfmf_oracle_total_sweeps.argtypes = [_I64, _P, _P]
        L.rfmf_oracle_total_sweeps.restype = _U64
        L.rfmf_oracle_max_threads.argtypes = []
        L.rfmf_oracle_max_threads.restype = ct.c_int
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data if a is not None else None


def philox_block(seed, step, block):
    out = np.zeros(4, np.uint32)
    lib().rfmf_oracle_philox_block(seed % 2**64, step, block, _ptr(out))
    return out


def gumbel(r11):
    return lib().rfmf_oracle_gumbel(r11)


def beta_fixed(step, t0):
    return lib().rfmf_oracle_beta_fixed(step, t0)


def score_safe_int32(total_steps, t0, B):
    return bool(lib().rfmf_oracle_score_safe_int32(total_steps, t0, B))


def max_weighted_degree(g):
    return lib().rfmf_oracle_max_weighted_degree(g.n, _ptr(g.offsets), _ptr(g.weight))


def cut_value(g, spin):
    spin = np.ascontiguousarray(spin, np.int8)
    return lib().rfmf_oracle_cut_value(g.n, _ptr(g.offsets), _ptr(g.col), _ptr(g.weight),
                                       _ptr(spin))


def initial_spins(seed, n):
    out = np.zeros(n, np.int8)
    lib().rfmf_oracle_initial_spins(seed % 2**64, n, _ptr(out))
    return out


def total_sweeps(phases, iters):
    ph = np.asarray(phases, np.uint64)
    it = np.asarray(iters, np.uint64)
    return int(lib().rfmf_oracle_total_sweeps(len(ph), _ptr(ph), _ptr(it)))


def max_threads():
    return lib().rfmf_oracle_max_threads()


def anneal(g, init_spins, t0s, solver_seeds, phases, iters, sweep_begin=0,
           sweep_end=None, best_spins=None, cur_vals=None, best_vals=None,
           trace=False, nthreads=0):
    """Run C chains over [sweep_begin, sweep_end) of the schedule.

    g: object with n, offsets (uint32), col (int32), weight (int32).
    init_spins: (C, n) int8 state at sweep_begin (copied).  For a window that
    does not start at 0, pass the carried best_spins/cur_vals/best_vals too.
    Returns dict(end_spins, best_spins, cur_vals, best_vals[, trace]).
    """
    spins = np.array(init_spins, np.int8, copy=True, order="C")
    C = spins.shape[0]
    n = g.n
    assert spins.shape == (C, n)
    ph = np.ascontiguousarray(phases, np.uint64)
    it = np.ascontiguousarray(iters, np.uint64)
    total = total_sweeps(ph, it)
    if sweep_end is None:
        sweep_end = total
    best = (spins.copy() if best_spins is None
            else np.array(best_spins, np.int8, copy=True, order="C"))
    if cur_vals is None:
        cur = np.array([cut_value(g, spins[c]) for c in range(C)], np.int64)
    else:
        cur = np.array(cur_vals, np.int64, copy=True)
    bestv = cur.copy() if best_vals is None else np.array(best_vals, np.int64, copy=True)
    t0a = np.ascontiguousarray(t0s, np.float64)
    sd = np.array([int(s) % 2**64 for s in solver_seeds], np.uint64)
    span = max(int(sweep_end) - int(sweep_begin), 0)
    tr = np.zeros((C, span), np.int64) if trace else None
    rc = lib().rfmf_oracle_anneal_window(
        n, _ptr(g.offsets), _ptr(g.col), _ptr(g.weight), C, _ptr(t0a), _ptr(sd),
        len(ph), _ptr(ph), _ptr(it), int(sweep_begin), int(sweep_end),
        _ptr(spins), _ptr(best), _ptr(cur), _ptr(bestv), _ptr(tr), int(nthreads))
    if rc != 0:
        raise RuntimeError("oracle anneal failed")
    out = dict(end_spins=spins, best_spins=best, cur_vals=cur, best_vals=bestv)
    if trace:
        out["trace"] = tr
    return out


def default_threads():
    return int(os.environ.get("OMP_NUM_THREADS", "0")) or max_threads()
