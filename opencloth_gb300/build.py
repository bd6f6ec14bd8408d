"""Build the native library ``libopencloth_gb.so`` in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into
``opencloth_gb300/_build/libopencloth_gb.so``.  Rebuilds only when a source, a header
or this file is newer than the library.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libopencloth_gb.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false keeps every FP32 multiply and add separately rounded, as the
# reference's scalar code rounds them; division and sqrt stay IEEE (no fast math).
# -ffp-contract=off does the same for host code (the lattice builder), where gcc on
# aarch64 would otherwise fuse multiply-adds.
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-Xcompiler", "-fno-strict-aliasing", "-I", str(INCLUDE), "-I", str(CSRC),
]
# The adjoint kernels differentiate the step; they are checked against finite differences
# and an FP64 adjoint, not against the reference's rounding sequence, so their unit
# contracts multiply-adds and uses the hardware's approximate division and square root.
GRADIENT_FLAGS = ["--fmad=true", "-prec-div=false", "-prec-sqrt=false"]
GRADIENT_SOURCES = {"oc_adjoint.cu"}
SOURCES = ["oc_kernels.cu", "oc_resident.cu", "oc_adjoint.cu", "oc_api.cu", "oc_topology.cpp", "oc_noalloc.cu",
           "oc_coupled.cu", "oc_interact.cu", "oc_bsr.cu"]


def _nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda) / "bin" / "nvcc"
    return str(cand) if cand.exists() else "nvcc"


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = [CSRC / f for f in os.listdir(CSRC)] + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.is_file())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src: str) -> Path:
        obj = BUILD / (src + ".o")
        lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
        flags = NVCC_FLAGS
        if src in GRADIENT_SOURCES:
            flags = [f for f in NVCC_FLAGS if f != "--fmad=false"] + GRADIENT_FLAGS
        cmd = [nvcc] + flags + lang + ["-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
        if verbose and res.stderr.strip():
            print(res.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
