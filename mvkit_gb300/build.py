"""Builds libmvkit_gb300.so in-tree (mvkit_gb300/_lib/) with nvcc for sm_103a.

Translation units compile in parallel; host code is compiled with
-ffp-contract=off so the FP64 model build and query planning round exactly
as the reference (x86-64 and aarch64 alike).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libmvkit_gb300.so"
# the reference-signature C layer (include/mvkit_gb300_mv.h), linked against LIB
MV_LIB = OUT / "libmvkit_gb300_mv.so"
SOURCES = ["ncc_kernels.cu", "ncc_tc.cu", "ncc_api.cpp", "ncc_model.cpp", "ncc_persist.cpp", "ncc_build.cu", "ncc_noalloc.cu"]
MV_SOURCES = ["mv_objects.cpp", "mv_ncc.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found: the CUDA extension cannot be built")


def _flags(src: str) -> list[str]:
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
              "-I", str(PKG.parent / "include")]
    if src.endswith(".cu"):
        return ARCH + common + ["--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
    return common + ["-x", "c++"]


def build(verbose: bool = False, force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    deps = ([CSRC / s for s in SOURCES + MV_SOURCES] + list(CSRC.glob("*.h")) +
            list((PKG.parent / "include").glob("*.h")))
    if (LIB.exists() and MV_LIB.exists() and not force and
            all(d.stat().st_mtime <= min(LIB.stat().st_mtime, MV_LIB.stat().st_mtime) for d in deps)):
        return LIB
    cc = nvcc()

    def compile_one(src: str) -> Path:
        obj = OUT / (src + ".o")
        cmd = [cc, *_flags(src), "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(len(SOURCES) + len(MV_SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES + MV_SOURCES))
    link = [cc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs[:len(SOURCES)]), "-lcudart"]
    mv_link = ["g++", "-shared", "-o", str(MV_LIB), *map(str, objs[len(SOURCES):]), f"-L{OUT}", "-lmvkit_gb300",
               "-Wl,-rpath,$ORIGIN", "-Wl,--no-undefined"]
    for cmd in (link, mv_link):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
