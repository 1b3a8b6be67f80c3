"""Drop-in boundary: the reference's own main.cu and host sources, compiled
unchanged, link against include/rfmf_annealgpu.hpp + librfmf.so in place of
src/anneal_kernels.cu.  Runs only where the reference checkout exists; on a
machine without a GPU the binary must stop with the reference-style error
message from the device call, after the host-side setup banner."""
import shutil
import subprocess

import pytest

from conftest import REFERENCE, ROOT


@pytest.mark.skipif(not (REFERENCE / "main.cu").exists(), reason="reference sources absent")
def test_reference_main_links_against_shim(rfmf, tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    lib = rfmf.lib()._name
    libdir = str((ROOT / "rfmf_gb300" / "_build"))
    (tmp_path / "shim.cpp").write_text('#include "anneal_gpu.cuh"\n#include "rfmf_annealgpu.hpp"\n')
    src = REFERENCE / "src"
    cmd = ["g++", "-std=c++17", "-O1", f"-I{src}", f"-I{REFERENCE}", f"-I{ROOT / 'include'}",
           "-x", "c++", str(REFERENCE / "main.cu"), str(tmp_path / "shim.cpp"),
           str(src / "host_common.cpp"), str(src / "max_cut.cpp"), str(src / "read_gset.cpp"),
           str(src / "graph.cpp"), f"-L{libdir}", "-lrfmf", f"-Wl,-rpath,{libdir}",
           "-o", str(tmp_path / "main_rfmf")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    assert lib
    run = subprocess.run([str(tmp_path / "main_rfmf"), str(REFERENCE / "Gset" / "G11"),
                          "--seeds", "1,2", "--t0s", "105,90", "--phases", "8,4",
                          "--iters", "10,10"], capture_output=True, text=True, timeout=120)
    assert "Chains: 2" in run.stderr
    import torch
    if torch.cuda.is_available():
        assert run.returncode == 0 and "summary: chains: 2" in run.stdout
    else:
        assert run.returncode != 0 and "rfmf_context_create failed" in run.stderr
