"""rfmf_gb300: GB300-native (sm_103a) RFMF annealer for weighted MAX-CUT.

The compute path is librfmf.so (hand-written CUDA + C++ host driver behind the
C ABI of include/rfmf.h); this package loads it through ctypes and mirrors the
reference's interface in Python.  There is no CPU fallback.
"""
from ._lib import BatchPlan, LaunchConfig, RfmfError, lib
from .api import (SOLVER_SEED_OFFSET, AnnealResult, Batch, Context, DeviceGraph, Server, anneal_gpu,
                  autotune,
                  beta_fixed, beta_tables, cut_value, debug_fail_host_alloc, debug_plan_items,
                  initial_spins,
                  make_config,
                  max_weighted_degree, parse_gset, score_safe_int32, solver_seed, total_steps,
                  version)
from .graphs import (CsrGraph, csr_from_edges, erdos_renyi, erdos_renyi_degree, erdos_renyi_sparse,
                     planar_like,
                     random_tree, read_gset, torus)

__all__ = [
    "BatchPlan", "LaunchConfig", "RfmfError", "lib", "SOLVER_SEED_OFFSET", "AnnealResult", "Batch",
    "Context", "DeviceGraph", "Server", "anneal_gpu", "beta_fixed", "beta_tables", "cut_value",
    "debug_fail_host_alloc", "debug_plan_items", "autotune",
    "initial_spins", "make_config", "max_weighted_degree", "parse_gset", "score_safe_int32", "solver_seed",
    "total_steps", "version", "CsrGraph", "csr_from_edges", "erdos_renyi",
    "erdos_renyi_degree", "erdos_renyi_sparse", "planar_like", "random_tree", "read_gset", "torus",
]
