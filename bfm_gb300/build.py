"""Build the GPU-backed libbfm.so in-tree (sm_103a only).

    python -m bfm_gb300.build            # -> bfm_gb300/lib/libbfm.so

CUDA sources go through nvcc with one -gencode (compute_103a -> sm_103a);
host C through gcc with -ffp-contract=off (gcc fuses multiply-adds by
default on aarch64, which would change the reference's rounding).  The CUDA
runtime is linked statically, so the library needs only the driver.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "lib"
BUILD_DIR = PKG / "_build"
LIB = OUT_DIR / "libbfm.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr"]
CC_FLAGS = ["-O2", "-fPIC", "-std=gnu11", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def sources() -> tuple[list[Path], list[Path]]:
    return sorted(CSRC.glob("*.cu")), sorted(CSRC.glob("*.c"))


def build(force: bool = False, verbose: bool = False) -> Path:
    cu, c = sources()
    deps = cu + c + sorted(INCLUDE.rglob("*.h")) + sorted(CSRC.glob("*.h")) + [Path(__file__)]
    if not force and LIB.exists() and (OUT_DIR / "libbfm.so.1").exists() and \
            LIB.stat().st_mtime > max(p.stat().st_mtime for p in deps):
        return LIB
    BUILD_DIR.mkdir(exist_ok=True)
    OUT_DIR.mkdir(exist_ok=True)
    nvcc = _nvcc()
    cc = os.environ.get("CC", "gcc")
    # the CUDA toolkit's headers for the host C files too (NVTX ranges)
    cuda_inc = Path(nvcc).resolve().parent.parent / "include"
    inc = [f"-I{INCLUDE}", f"-I{CSRC}", f"-I{cuda_inc}"]
    jobs = []
    for src in cu:
        obj = BUILD_DIR / (src.stem + ".cu.o")
        jobs.append(([nvcc, *ARCH, *NVCC_FLAGS, *inc, "-c", str(src), "-o", str(obj)], obj))
    for src in c:
        obj = BUILD_DIR / (src.stem + ".c.o")
        jobs.append(([cc, *CC_FLAGS, *inc, "-c", str(src), "-o", str(obj)], obj))
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        for cmd, _ in jobs:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
        list(ex.map(lambda j: _run(j[0]), jobs))
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *[str(o) for _, o in jobs], "-Xlinker", "-Bsymbolic",
          "-Xlinker", "-soname=libbfm.so.1", "-lpthread", "-lm", "-ldl"])
    os.replace(tmp, LIB)
    # the soname the link records (libbfm.so.1, as the reference's SOVERSION 1),
    # for programs linked with -lbfm against this directory
    so1 = OUT_DIR / "libbfm.so.1"
    if so1.is_symlink() or so1.exists():
        so1.unlink()
    so1.symlink_to(LIB.name)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
