"""Host-side helpers of librfmf.so (rfmf_gb300/csrc/rfmf_host.h), compiled
into small harnesses with g++ (pure host code: no GPU, no CUDA call).

* Spin packing (pack_spins, unpack_spins): the conversion every entry point
  applies between the caller's int8 spins (>= 0 is +1) and the kernel's bit
  words (bit v = spin +1), checked on random and edge-case inputs against the
  bit-at-a-time definition, at every length 1..70 and at the graph sizes of
  the workloads (n = 800 .. 20000).
* The request server's admission rule (admits) and a request's device
  footprint (request_device_bytes), which max_device_bytes is counted in.
"""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

HARNESS = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "rfmf_host.h"
int rfmf::fail(int c, const char*, ...) { return c; }
int rfmf::set_last_error(int c, const char*) { return c; }
using namespace rfmf;
static int check(int64_t n, int mode) {
    std::vector<int8_t> sp(n + 8);
    for (int64_t v = 0; v < n; ++v) {
        const int r = rand();
        sp[v] = mode == 0 ? ((r & 1) ? 1 : -1)           // +-1
              : mode == 1 ? static_cast<int8_t>(r % 256 - 128)   // any int8: >= 0 is +1
              : mode == 2 ? 1 : -1;                        // all +1 / all -1
    }
    const int64_t words = (n + 31) / 32;
    std::vector<uint32_t> ref(words + 1, 0u), got(words + 1, 0xA5A5A5A5u);
    for (int64_t v = 0; v < n; ++v) if (sp[v] >= 0) ref[v >> 5] |= 1u << (v & 31);
    pack_spins(sp.data(), n, got.data());
    for (int64_t w = 0; w < words; ++w) if (ref[w] != got[w]) return 1;
    if (got[words] != 0xA5A5A5A5u) return 2;               // nothing past the last word
    std::vector<int8_t> out(n + 8, 42);
    unpack_spins(ref.data(), n, out.data());
    for (int64_t v = 0; v < n; ++v)
        if (out[v] != (((ref[v >> 5] >> (v & 31)) & 1u) ? 1 : -1)) return 3;
    for (int k = 0; k < 8; ++k) if (out[n + k] != 42) return 4;   // nothing past n
    return 0;
}
int main() {
    srand(7);
    std::vector<int64_t> ns;
    for (int64_t n = 1; n <= 70; ++n) ns.push_back(n);
    for (int64_t n : {255, 256, 257, 800, 2000, 3000, 5000, 10000, 19881, 20000}) ns.push_back(n);
    for (int64_t n : ns)
        for (int mode = 0; mode < 4; ++mode)
            if (int rc = check(n, mode)) { printf("FAIL n=%lld mode=%d rc=%d\n", (long long)n, mode, rc); return 1; }
    printf("ok %zu lengths\n", ns.size());
    return 0;
}
"""


ADMISSION = r"""
#include <cstdio>
#include "rfmf_host.h"
int rfmf::fail(int c, const char*, ...) { return c; }
int rfmf::set_last_error(int c, const char*) { return c; }
using namespace rfmf;
int main() {
    const int64_t T = int64_t(1) << 40;
    int bad = 0;
    // an idle server admits the queue head whatever its size
    bad |= !admits(0, 0, 1 << 20, T, 8, 1000) << 0;
    // no byte limit: only the chain cap counts
    bad |= !admits(10, T, 90, T, 100, 0) << 1;
    bad |= admits(10, 0, 91, 0, 100, 0) << 2;
    // byte limit: inclusive, and both limits must hold
    bad |= !admits(1, 500, 1, 500, 100, 1000) << 3;
    bad |= admits(1, 500, 1, 501, 100, 1000) << 4;
    bad |= admits(99, 0, 2, 10, 100, 1000) << 5;
    printf("%d %zu %lld %lld\n", bad, sizeof(DevChain),
           (long long)request_device_bytes(2, 3, 5, 8), (long long)request_device_bytes(256, 625, 273000, 0));
    return 0;
}
"""


def _cuda_include():
    for base in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if base and os.path.exists(os.path.join(base, "include", "cuda_runtime.h")):
            return os.path.join(base, "include")
    return None


def test_pack_unpack_match_bitwise_definition(tmp_path):
    r = _build_run(tmp_path, HARNESS, "pack")
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")

def _build_run(tmp_path, code, name):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip("g++ or the CUDA headers are missing")
    src = tmp_path / (name + ".cpp")
    src.write_text(code)
    exe = tmp_path / name
    subprocess.run([cxx, "-O2", "-std=c++17", "-Wall", "-I", str(ROOT / "rfmf_gb300" / "csrc"),
                    "-I", inc, str(src), "-o", str(exe)], check=True, capture_output=True)
    return subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)


def test_server_admission_rule_and_footprint(tmp_path):
    r = _build_run(tmp_path, ADMISSION, "admission")
    assert r.returncode == 0, r.stderr
    bad, chain_rec, small, large = (int(x) for x in r.stdout.split())
    assert bad == 0, f"admission cases failed (bit mask {bad:#x})"
    # 2 chains x 3 words: bits + best 2 x 24 B, 5 runs: 40 + 20 B, 8 phases: 32 + 64 B
    assert small == 2 * 24 + 40 + 20 + 32 + 64 + 2 * chain_rec
    # empty schedule and short buffers take the 16-byte minimum
    assert large == 2 * 256 * 625 * 4 + 273000 * 12 + 16 + 16 + 256 * chain_rec
