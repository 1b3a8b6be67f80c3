"""Run the reference's own kernel (oracle/_ref/anneal_kernels.cubin) on the GPU.

TEST INFRASTRUCTURE ONLY.  The launch choices follow the reference's host
code: sWidth from B (main.cu:51), corr from mean degree (main.cu:41-45), the
int32 gate at min(t0s) over the sum of all iters (src/anneal_kernels.cu:
633-639), threads per block from src/tuning.hpp via src/anneal_kernels.cu:
641-662, beta tables from buildBetaRunTables over the same total.
"""
import ctypes as ct
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "anneal_kernels.cubin"
LIB = HERE / "_build" / "librefgpu.so"
_P, _I64 = ct.c_void_p, ct.c_int64
_lib = None


def available():
    return CUBIN.exists()


def lib():
    global _lib
    if _lib is None:
        import subprocess
        if not LIB.exists():
            subprocess.run(["make", "-C", str(HERE), "-s", "_build/librefgpu.so"], check=True)
        L = ct.CDLL(str(LIB))
        L.refgpu_run.argtypes = [ct.c_char_p, ct.c_int, ct.c_int, ct.c_int, ct.c_int, _I64, _P, _P,
                                 _P, _I64, _P, _P, _I64, _P, _P, _P, _P, _I64, _P, _P, _P, _P,
                                 _P, _P, _P, _P, ct.c_char_p, ct.c_int]
        L.refgpu_run.restype = ct.c_int
        _lib = L
    return _lib


def reference_choices(g, C, t0s, iters, sm_count):
    import oracle as ora
    B = ora.max_weighted_degree(g)
    total = int(sum(int(x) for x in iters))
    mean_deg = 2.0 * g.m / g.n if g.n else 0.0
    warp = mean_deg >= 8.0
    if C > sm_count:
        tpb = 512 if g.n > 16384 else 256
    elif warp:
        tpb = 1024
    else:
        tpb = 512 if g.n <= 1024 else 896
    return dict(B=B, s64=B > 2**31 - 1, packed=ora.score_safe_int32(total, min(t0s), B),
                corr_warp=warp, tpb=tpb, total=total)


def run(g, init_spins, t0s, solver_seeds, phases, iters, sm_count, tpb=None):
    import oracle as ora
    import rfmf_gb300 as R
    init = np.ascontiguousarray(init_spins, np.int8)
    C = init.shape[0]
    ch = reference_choices(g, C, t0s, iters, sm_count)
    end, val, off = R.beta_tables(t0s, ch["total"])
    cut0 = np.array([ora.cut_value(g, init[c]) for c in range(C)], np.int64)
    ph = np.ascontiguousarray(phases, np.uint64)
    it = np.ascontiguousarray(iters, np.uint64)
    sd = np.array([int(s) % 2**64 for s in solver_seeds], np.uint64)
    e_sp = np.zeros_like(init)
    b_sp = np.zeros_like(init)
    cur = np.zeros(C, np.int64)
    best = np.zeros(C, np.int64)
    ms = ct.c_float(0)
    used = ct.c_int(0)
    err = ct.create_string_buffer(256)
    rc = lib().refgpu_run(str(CUBIN).encode(), int(ch["s64"]), int(ch["packed"]),
                          int(ch["corr_warp"]), int(tpb or ch["tpb"]), g.n,
                          g.offsets.ctypes.data, g.col.ctypes.data, g.weight.ctypes.data, C,
                          init.ctypes.data, cut0.ctypes.data, len(end), end.ctypes.data,
                          val.ctypes.data, off.ctypes.data, sd.ctypes.data, len(ph),
                          ph.ctypes.data, it.ctypes.data, e_sp.ctypes.data, b_sp.ctypes.data,
                          cur.ctypes.data, best.ctypes.data, ct.byref(ms), ct.byref(used), err,
                          256)
    if rc != 0:
        raise RuntimeError(f"reference kernel: {err.value.decode()}")
    return dict(end_spins=e_sp, best_spins=b_sp, cur_vals=cur, best_vals=best, ms=ms.value,
                tpb=used.value, choices=ch)
