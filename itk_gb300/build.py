"""Builds the in-tree CUDA library ``itk_gb300/_lib/libitk_gb300.so`` for sm_103a.

Each translation unit under ``itk_gb300/csrc`` is compiled by nvcc in
parallel (one ``-gencode``, ``-lineinfo``) and linked into one shared
library; nothing is installed outside the repository.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(OUT_DIR, "libitk_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FMA contraction (aarch64 g++ contracts a*b+c by default), so host-side
# FP64 geometry and transform constants round like the reference on every host ISA
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc_path() -> str:
    cand = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cand, "bin", "nvcc")
    if os.path.exists(p):
        return p
    w = shutil.which("nvcc")
    if not w:
        raise RuntimeError("nvcc not found: set CUDA_HOME")
    return w


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "itk_gb300.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = nvcc_path()
    cuda_home = os.path.dirname(os.path.dirname(nvcc))
    inc = ["-I", os.path.join(cuda_home, "include", "cccl"), "-I", os.path.join(HERE, "..", "include")]
    flags = NVCC_FLAGS + ARCH + inc + list(extra_flags or [])

    def compile_one(src):
        obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
        cmd = [nvcc, "-c", src, "-o", obj] + flags
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
