"""Builds librustracer_cuda.so in-tree: every CUDA translation unit for sm_103a plus the host C++.

Usage: python -m rustracer_gb300.build [--force] [--verbose]

nvcc cross-compiles without a GPU.  Objects go to rustracer_gb300/_build/, the shared library to
rustracer_gb300/librustracer_cuda.so and the same objects as a static archive to
rustracer_gb300/librustracer_cuda.a (all git-ignored; a static link also needs the CUDA runtime:
-lcudart_static -lstdc++ -lpthread -ldl -lrt).  Translation units compile in parallel and are rebuilt
when a source or header is newer than the object.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "librustracer_cuda.so"
STATIC_LIB = PKG / "librustracer_cuda.a"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: a*b+c is rounded twice, as the WGSL shaders' separate multiply and add are.
# IEEE division and square root (no --use_fast_math).
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-warn-spills",
              "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librustracer_cuda.so")


def _cuda_lib_dir(nvcc: str) -> Path:
    root = Path(nvcc).resolve().parent.parent
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        if (root / sub / "libcudart_static.a").exists() or (root / sub / "libcudart.so").exists():
            return root / sub
    return root / "lib64"


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return t < src.stat().st_mtime or t < newest_header


# The image-space kernels (denoise, composite + tonemap) are compiled with FMA contraction: their
# parity tests compare within 1e-5 relative (denoise) and +-1 rgba8 step (tonemap); composite stays
# bit-exact because its mix is written with explicitly rounded products and sum (__fmul_rn /
# __fadd_rn, which are never contracted).
FMAD_ON = {"k_image.cu"}


def _compile(nvcc: str, src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.name + ".o")
    if src.suffix == ".cu":
        flags = [f if not (src.name in FMAD_ON and f == "--fmad=false") else "--fmad=true" for f in NVCC_FLAGS]
        cmd = [nvcc, *ARCH, *flags, "-c", str(src), "-o", str(obj)]
    else:
        cxx = shutil.which("g++") or "c++"
        cmd = [cxx, *CXX_FLAGS, "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compiling {src.name} failed:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr.strip():
        print(res.stderr, flush=True)
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
    srcs = sources()
    todo = [s for s in srcs if force or _stale(BUILD / (s.name + ".o"), s, newest_header)]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda s: _compile(nvcc, s, verbose), todo))
    objs = [BUILD / (s.name + ".o") for s in srcs]
    if force or todo or not LIB.exists() or any(LIB.stat().st_mtime < o.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static",
               "-L" + str(_cuda_lib_dir(nvcc)), "-lpthread", "-ldl", "-lrt"]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"linking librustracer_cuda.so failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    if force or todo or not STATIC_LIB.exists() or any(STATIC_LIB.stat().st_mtime < o.stat().st_mtime for o in objs):
        tmp_a = STATIC_LIB.with_suffix(".a.tmp")
        if tmp_a.exists():
            tmp_a.unlink()
        res = subprocess.run([shutil.which("ar") or "ar", "rcs", str(tmp_a), *map(str, objs)], capture_output=True,
                             text=True)
        if res.returncode != 0:
            raise RuntimeError(f"archiving librustracer_cuda.a failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp_a, STATIC_LIB)
    return LIB


def cuda_lib_dir() -> Path:
    """The CUDA toolkit's library directory (libcudart_static.a for a static link)."""
    return _cuda_lib_dir(_nvcc())


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build(force=a.force, verbose=a.verbose))
    return 0


if __name__ == "__main__":
    sys.exit(main())
