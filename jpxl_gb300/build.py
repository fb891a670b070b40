"""Builds the sm_103a library ``libjpxlg.so`` in-tree (jpxl_gb300/_lib/).

Every translation unit is compiled by nvcc with one ``-gencode`` for
compute_103a/sm_103a, relocatable device code (the DCT constant tables are
shared across units; the tensor-core unit is whole-program code, see
WHOLE_PROGRAM_UNITS), ``-fmad=false`` (the reference never contracts a*b+c)
and ``-ffp-contract=off`` for the host table code.  Units compile in
parallel; a unit is rebuilt only when a source or header is newer than its
object.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "_lib"
OBJ_DIR = OUT_DIR / "obj"
LIB = OUT_DIR / "libjpxlg.so"
INCLUDE = HERE.parent / "include"

UNITS = ["tables.cu", "k_encode.cu", "k_cover.cu", "k_render.cu", "k_ssim.cu", "k_blur.cu",
         "jpxlg_api.cu", "entropy.cu", "codestream.cu", "k_tc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = [
    "-O3",
    "-std=c++17",
    "-rdc=true",
    "-lineinfo",
    "-fmad=false",
    "-prec-div=true",
    "-prec-sqrt=true",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off,-fno-fast-math",
    "-Xptxas",
    "-warn-spills",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build libjpxlg.so")


def _newest_header() -> float:
    heads = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return max(p.stat().st_mtime for p in heads)


# Units compiled as whole-program device code: the tensor-core unit, whose
# tcgen05 sequence gave wrong accumulators when built as relocatable device
# code (it refers to no device symbol of another unit).
WHOLE_PROGRAM_UNITS = {"k_tc.cu"}


def _compile(unit: str, extra: list[str]) -> Path:
    src = CSRC / unit
    obj = OBJ_DIR / (unit + ".o")
    if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, _newest_header()):
        return obj
    flags = [f for f in FLAGS if not (unit in WHOLE_PROGRAM_UNITS and f == "-rdc=true")]
    cmd = [nvcc(), *ARCH, *flags, *extra, "-I", str(CSRC), "-I", str(INCLUDE), "-c", str(src),
           "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {unit}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compiles (incrementally) and links ``libjpxlg.so``; returns its path."""
    extra = extra or []
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS)) as pool:
        objs = list(pool.map(lambda u: _compile(u, extra), UNITS))
    if not LIB.exists() or LIB.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-rdc=true", "-o", str(LIB), *map(str, objs),
               "-Xcompiler", "-fPIC", "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
