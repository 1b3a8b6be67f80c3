"""The Python mirrors of the C ABI's structs (rfmf_gb300/_lib.py) have the
layout include/rfmf.h gives them: a C program generated from the ctypes
field lists, compiled with the system C compiler against the header,
prints every field's offset and size and every struct's size, and each must
equal ctypes' own.  A field missing from the header fails the compile; one
missing from the mirror, or reordered, or of another width, fails the
comparison.  Host only: nothing is loaded or launched."""
import ctypes as ct
import shutil
import subprocess

import pytest

from conftest import ROOT

MIRRORS = {
    "rfmf_launch_config": "LaunchConfig",
    "rfmf_batch_plan": "BatchPlan",
    "rfmf_server_config": "ServerConfig",
    "rfmf_request_status": "RequestStatus",
    "rfmf_server_stats": "ServerStats",
}


def test_ctypes_mirrors_match_header_layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    from rfmf_gb300 import _lib
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "rfmf.h"', "int main(void) {"]
    expect = []
    for cname, pyname in MIRRORS.items():
        py = getattr(_lib, pyname)
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        expect.append(f"{cname} sizeof {ct.sizeof(py)}")
        for fname, ftype in py._fields_:
            lines.append(f'  printf("{cname}.{fname} %zu %zu\\n", offsetof({cname}, {fname}), '
                         f'sizeof((({cname}*)0)->{fname}));')
            expect.append(f"{cname}.{fname} {getattr(py, fname).offset} {ct.sizeof(ftype)}")
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c99", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    assert [g for g in got if g] == expect
