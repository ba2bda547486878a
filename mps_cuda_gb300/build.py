"""Builds libmps_gb300.so (the C-ABI CUDA library) in-tree with nvcc for sm_103a.

Translation units are compiled in parallel and linked with `nvcc -shared`; the output lands next
to this file so that the package loads it without any install step.  Rebuilds only when a source
is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
LIB = HERE / "libmps_gb300.so"
BUILD = HERE / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden"]
# Extra nvcc flags (e.g. -DMPSG_B_AP=8 to retune a neighbour loop); a change needs build(force=True).
NVCC_FLAGS += os.environ.get("MPS_GB300_NVCC_FLAGS", "").split()
SOURCES = ["sort.cu", "sph.cu", "api.cu", "ops.cu", "noalloc.cu", "mesh.cu", "adjoint.cu", "scene.cpp"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libmps_gb300.so")
    return cand


def _needs_build() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def _compile(src: str, verbose: bool) -> Path:
    out = BUILD / (src + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", "-c", str(CSRC / src), "-o", str(out)]
    if src.endswith(".cpp"):
        # host code: no floating-point contraction, so x86 and Arm give the same bits
        cmd = [nvcc(), "-x", "c++", *NVCC_FLAGS, "-Xcompiler", "-ffp-contract=off", f"-I{INCLUDE}", "-c",
               str(CSRC / src), "-o", str(out)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return out


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles every translation unit for sm_103a and links libmps_gb300.so."""
    if not force and not _needs_build():
        return LIB
    BUILD.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
