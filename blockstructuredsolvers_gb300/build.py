"""Build recipe for the sm_103a C-ABI library ``libbss_gb300.so``.

nvcc compiles each translation unit of ``csrc/`` for exactly one target,
``-gencode arch=compute_103a,code=sm_103a``, in parallel, then links one
shared library in this package directory (in-tree, so the process that
loads it is visible to whoever inspects loaded objects).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbss_gb300.so")
SOURCES = ["k_f32.cu", "k_f64.cu", "k_mixed.cu", "bss_api.cu", "bss_upload.cu", "bss_noalloc.cu", "bss_batch.cu", "bss_server.cu", "bss_tune.cu", "bss_cpu.cu", "bss_diag.cu", "bss_refalgo.cu", "bss_sparse.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "bss.h"))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [cc, *ARCH, *FLAGS, *(extra or []), "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"--- {src} ---\n{out.decode(errors='replace')}")
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call([cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcublas", "-lcusolver", "-lcusparse"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
