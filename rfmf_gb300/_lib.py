"""ctypes bindings onto librfmf.so (the C ABI of include/rfmf.h).

The library is the product; this module only loads it and declares the
signatures.  Loading fails loudly when the library is missing: there is no
CPU fallback anywhere in the package.
"""
import ctypes as ct
import os
import pathlib

from . import build as _build

_P = ct.c_void_p
_I64 = ct.c_int64
_U64 = ct.c_uint64
_I32 = ct.c_int32

# (name, restype, argtypes) for every symbol the C headers (include/rfmf.h and
# the testing aids of include/rfmf_testing.h) declare.
SIGNATURES = [
    ("rfmf_version", ct.c_char_p, []),
    ("rfmf_last_error", ct.c_char_p, []),
    ("rfmf_context_create", ct.c_int, [ct.c_int, _P]),
    ("rfmf_context_destroy", ct.c_int, [_P]),
    ("rfmf_context_info", ct.c_int, [_P, _P, _P]),
    ("rfmf_context_stream", ct.c_int, [_P, _P]),
    ("rfmf_context_beta_cache", ct.c_int, [_P, _P, _P, _P]),
    ("rfmf_graph_create", ct.c_int, [_P, _I64, _P, _P, _P, _P]),
    ("rfmf_graph_destroy", ct.c_int, [_P]),
    ("rfmf_csr_validate", ct.c_int, [_I64, _P, _P, _P, _P]),
    ("rfmf_graph_info", ct.c_int, [_P, _P, _P, _P]),
    ("rfmf_total_steps", _I64, [_I64, _P]),
    ("rfmf_beta_fixed", _I32, [_U64, ct.c_double]),
    ("rfmf_score_safe_int32", ct.c_int, [_I64, ct.c_double, _I64]),
    ("rfmf_max_weighted_degree", _I64, [_I64, _P, _P]),
    ("rfmf_cut_value", _I64, [_I64, _P, _P, _P, _P]),
    ("rfmf_initial_spins", None, [_U64, _I64, _P]),
    ("rfmf_beta_tables", ct.c_int, [_P, _I64, _I64, _P, _P, _P, _I64, _P]),
    ("rfmf_anneal", ct.c_int, [_P, _P, _I64, _I64, _P, _P, _I64, _P, _P, _P, _P,
                               _P, _P, _P, _P, _P]),
    ("rfmf_batch_create", ct.c_int, [_P, _I64, _P, _P, _P, _P, _I64, _P, _P, _P, _P]),
    ("rfmf_batch_run", ct.c_int, [_P, _U64]),
    ("rfmf_batch_run_graph", ct.c_int, [_P, _U64, ct.c_int, ct.c_int]),
    ("rfmf_batch_run_timed", ct.c_int, [_P, _U64, _P]),
    ("rfmf_batch_stats", ct.c_int, [_P, _P]),
    ("rfmf_batch_debug_set_cut", ct.c_int, [_P, _I64, _I64]),
    ("rfmf_batch_synchronize", ct.c_int, [_P]),
    ("rfmf_batch_read", ct.c_int, [_P, _P, _P, _P, _P, _P]),
    ("rfmf_batch_restore", ct.c_int, [_P, _I64, _P, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P,
                                      _P, _P]),
    ("rfmf_debug_fail_host_alloc", ct.c_int, [_I64]),
    ("rfmf_debug_plan_items", ct.c_int, [ct.c_int, _P, ct.c_int, ct.c_int, _P, _I64, _P]),
    ("rfmf_batch_info", ct.c_int, [_P, _P]),
    ("rfmf_autotune", ct.c_int, [_P, _I64, _P, _P, _P, _P, _I64, _P, _P, _U64, _P, _P, _P, _P,
                                 _P]),
    ("rfmf_batch_destroy", ct.c_int, [_P]),
    ("rfmf_anneal_noalloc", ct.c_int, [ct.c_int, _P, _I64, _P, _P, _I64, _I64, _P, _P, _I64,
                                       _P, _P, _P, _P, _I64, _P, _P, _P, _P, _P, _P]),
    ("rfmf_gset_header", ct.c_int, [ct.c_char_p, ct.c_size_t, _P, _P]),
    ("rfmf_gset_parse", ct.c_int, [ct.c_char_p, ct.c_size_t, ct.c_double, _I64, _P, _P, _P, _P,
                                   _P, _P]),
    ("rfmf_graph_from_edges", ct.c_int, [_P, _I64, _P, _P, _P, _P, _P]),
    ("rfmf_graph_orig_ids", ct.c_int, [_P, _P]),
    ("rfmf_graph_csr", ct.c_int, [_P, _P, _P, _P]),
    ("rfmf_batch_cuts", ct.c_int, [_P, ct.c_int, _P]),
    ("rfmf_batch_partitions", ct.c_int, [_P, ct.c_int, _P, _I64]),
    ("rfmf_server_create", ct.c_int, [_P, _P, _P]),
    ("rfmf_server_destroy", ct.c_int, [_P]),
    ("rfmf_submit", ct.c_int, [_P, _P, _I64, _P, _P, _I64, _P, _P, _P, _P]),
    ("rfmf_poll", ct.c_int, [_P, _U64, _P]),
    ("rfmf_wait", ct.c_int, [_P, _U64, ct.c_double, _P]),
    ("rfmf_result", ct.c_int, [_P, _U64, _P, _P, _P, _P]),
    ("rfmf_server_stats_get", ct.c_int, [_P, _P]),
    ("rfmf_cancel", ct.c_int, [_P, _U64]),
]


class LaunchConfig(ct.Structure):
    """rfmf_launch_config (mirrors gpu3::LaunchConfig plus tuning knobs)."""
    _fields_ = [("corr", ct.c_int), ("device", ct.c_int), ("s_width", ct.c_int),
                ("threads_per_chain", ct.c_int), ("score_path", ct.c_int),
                ("chains_per_cta", ct.c_int), ("csr_format", ct.c_int),
                ("gain_width", ct.c_int)]


class BatchPlan(ct.Structure):
    """rfmf_batch_plan."""
    _fields_ = [("nchains", ct.c_int64), ("total_sweeps", ct.c_uint64),
                ("threads_per_chain", ct.c_int), ("chains_per_cta", ct.c_int),
                ("grid", ct.c_int), ("items", ct.c_int), ("score64", ct.c_int),
                ("csr_format", ct.c_int), ("gain_width", ct.c_int), ("smem_bytes", ct.c_int),
                ("balanced", ct.c_int), ("launch_classes", ct.c_int), ("launches", ct.c_int64)]


class ServerConfig(ct.Structure):
    """rfmf_server_config."""
    _fields_ = [("window_sweeps", ct.c_uint64), ("max_chains", ct.c_int64),
                ("launch", LaunchConfig), ("max_device_bytes", ct.c_int64)]


class RequestStatus(ct.Structure):
    """rfmf_request_status."""
    _fields_ = [("state", ct.c_int), ("error", ct.c_int), ("sweeps_done", ct.c_uint64),
                ("sweeps_total", ct.c_uint64), ("submit_s", ct.c_double),
                ("start_s", ct.c_double), ("finish_s", ct.c_double)]


class ServerStats(ct.Structure):
    """rfmf_server_stats."""
    _fields_ = [("windows", ct.c_uint64), ("launches", ct.c_uint64),
                ("chain_sweeps", ct.c_uint64), ("busy_s", ct.c_double),
                ("kernel_s", ct.c_double), ("queued", ct.c_int64), ("running", ct.c_int64),
                ("done", ct.c_int64)]


REQUEST_STATES = {0: "queued", 1: "running", 2: "done", 3: "failed", 4: "cancelled"}

STATUS = {0: "RFMF_OK", 1: "RFMF_ERR_INVALID", 2: "RFMF_ERR_CUDA", 3: "RFMF_ERR_NOMEM",
          4: "RFMF_ERR_CAPACITY", 5: "RFMF_ERR_DEVICE", 6: "RFMF_ERR_BETA_RUNS"}


class RfmfError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def library_path():
    return pathlib.Path(os.environ.get("RFMF_LIB", str(_build.LIB)))


def lib(build_if_missing=True):
    """Load librfmf.so (building it first if absent and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists() and build_if_missing:
        _build.build()
    if not path.exists():
        raise RuntimeError(f"librfmf.so not found at {path}; run rfmf_gb300.build.build()")
    L = ct.CDLL(str(path))
    for name, res, args in SIGNATURES:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(code):
    if code != 0:
        raise RfmfError(code, lib().rfmf_last_error().decode(errors="replace"))
    return code
