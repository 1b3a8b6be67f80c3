"""Build librfmf.so (sm_103a) in-tree with nvcc.

The translation units compile in parallel and link into
rfmf_gb300/_build/librfmf.so.  No cmake, no torch extension machinery: the
library is plain C ABI over CUDA, so it builds the same on x86_64 and aarch64.
"""
import os
import pathlib
import shutil
import subprocess
import sys

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "librfmf.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "-I", str(INCLUDE), "-I", str(CSRC)]
SOURCES = ["rfmf_anneal.cu", "rfmf_driver.cpp", "rfmf_batch.cpp", "rfmf_noalloc.cu",
           "rfmf_server.cpp", "rfmf_ingest.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and pathlib.Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale():
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [pathlib.Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force=False, verbose=False, ptxas_verbose=False):
    """Compile if any source is newer than the library.  Returns the path."""
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    nv = nvcc()
    procs = []
    objs = []
    for src in SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        cmd = [nv] + ARCH + NVCC_FLAGS + ["-c", str(CSRC / src), "-o", str(obj)]
        if ptxas_verbose and src.endswith(".cu"):
            cmd += ["-Xptxas", "-v"]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                            text=True)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{out}")
        if verbose and out:
            sys.stdout.write(out)
    tmp = BUILD / "librfmf.so.tmp"
    link = [nv] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_verbose="-v" in sys.argv)
    print(LIB)
