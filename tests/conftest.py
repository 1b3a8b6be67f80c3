import os
import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

GOLDEN = ROOT / "tests" / "golden"
REFERENCE = pathlib.Path(os.environ.get("RFMF_REFERENCE", "/root/reference"))
REF_HOST_LIB = ROOT / "oracle" / "_ref" / "libref_host.so"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through librfmf.so)")
    config.addinivalue_line("markers", "slow: long CPU run, deselected unless asked for")


@pytest.fixture(scope="session")
def oracle():
    import oracle as ora
    ora.build()
    return ora


@pytest.fixture(scope="session")
def rfmf():
    import rfmf_gb300 as R
    from rfmf_gb300 import build as B
    B.build()
    return R


@pytest.fixture(scope="session")
def ctx(rfmf):
    c = rfmf.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def ref_host():
    """The reference's own host code (oracle/_ref), where it was built."""
    if not REF_HOST_LIB.exists():
        pytest.skip("oracle/_ref not built (needs the reference sources)")
    import ctypes as ct
    L = ct.CDLL(str(REF_HOST_LIB))
    P, I64, U64 = ct.c_void_p, ct.c_int64, ct.c_uint64
    L.ref_philox_block.argtypes = [U64, U64, U64, P]
    L.ref_gumbel.argtypes = [ct.c_uint32]
    L.ref_gumbel.restype = ct.c_int32
    L.ref_beta_fixed.argtypes = [U64, ct.c_double]
    L.ref_beta_fixed.restype = ct.c_int32
    L.ref_beta_tables.argtypes = [P, I64, I64, P, P, P, I64]
    L.ref_beta_tables.restype = I64
    L.ref_score_safe_int32.argtypes = [I64, ct.c_double, I64]
    L.ref_score_safe_int32.restype = ct.c_int
    L.ref_initial_spins.argtypes = [U64, I64, P]
    L.ref_gset_load.argtypes = [ct.c_char_p]
    L.ref_gset_load.restype = P
    for f in ("ref_gset_n", "ref_gset_m", "ref_gset_max_weighted_degree"):
        getattr(L, f).argtypes = [P]
        getattr(L, f).restype = I64
    L.ref_gset_copy.argtypes = [P, P, P, P]
    L.ref_gset_cut.argtypes = [P, P]
    L.ref_gset_cut.restype = I64
    L.ref_gset_free.argtypes = [P]
    return L


@pytest.fixture(scope="session")
def refgpu():
    """The reference's own kernel (oracle/_ref/anneal_kernels.cubin, built from
    its sources by oracle/build_ref.sh) launched through oracle/refgpu.py."""
    import refgpu as RG
    if not RG.available():
        pytest.skip("reference kernel cubin not built on this machine")
    return RG


def chains_for(g, seeds):
    """Initial spins (from raw seeds) and solver seeds, as setupSolver/main do."""
    import oracle as ora
    init = np.stack([ora.initial_spins(s, g.n) for s in seeds])
    solver = [(int(s) + 0xC2B2AE3D27D4EB4F) % 2**64 for s in seeds]
    return init, solver
