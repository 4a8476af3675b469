"""Builds libelpaso_gb300.so (CUDA sm_103a + host C++) in-tree.

Every translation unit in csrc/ is compiled in parallel with nvcc for
`-gencode arch=compute_103a,code=sm_103a` and linked into one shared
library with a plain C ABI (include/elpaso_gb300.h). No torch, no cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(os.path.dirname(HERE), "_build", "obj-" + __import__("platform").machine())
LIB_NAME = "libelpaso_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(
        os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp"))
    )


def _compile(nvcc: str, src: str, extra: list[str]) -> tuple[str, str]:
    obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(os.path.dirname(HERE), "include", "elpaso_gb300.h")
    ]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj, ""
    cmd = [
        nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp,-O3",
        "-c", src, "-o", obj,
    ] + extra
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{proc.stdout}\n{proc.stderr}")
    return obj, proc.stderr


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    """Compiles and links; returns the path of the shared library."""
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = nvcc_path()
    extra = list(extra or [])
    objs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, nvcc, s, extra) for s in sources()]
        for fu in futs:
            obj, log = fu.result()
            objs.append(obj)
            if verbose and log:
                print(log, file=sys.stderr)
    lib = os.path.join(OUT_DIR, LIB_NAME)
    tmp = lib + ".tmp"
    cmd = [nvcc, ARCH, "-shared", "-o", tmp] + objs + ["-Xcompiler", "-fopenmp", "-lcudart"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"link failed:\n{proc.stdout}\n{proc.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
