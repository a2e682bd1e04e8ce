"""Build recipe of the CUDA library (in-tree, no cmake).

    python -c "import axisem_gb300.build as b; b.build()"

compiles ``csrc/axg_api.cu`` and ``csrc/axg_plan.cpp`` for sm_103a into
``axisem_gb300/_build/libaxisem_gb300.so``.  The translation units are
compiled in parallel; a rebuild happens only when a source is newer than the
library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libaxisem_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include"),
          "-I", str(CSRC)]
CUDA_FLAGS = ARCH + ["-ftz=true", "-prec-div=true", "-prec-sqrt=true", "--expt-relaxed-constexpr"]

SOURCES = ["axg_api.cu", "axg_plan.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _deps() -> list[Path]:
    return [CSRC / s for s in SOURCES] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [
        ROOT / "include" / "axisem_gb300.h"]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    if not force and up_to_date():
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    extra = extra or []

    def compile_one(src: str) -> Path:
        obj = OUT / (src.replace(".", "_") + ".o")
        flags = COMMON + (CUDA_FLAGS if src.endswith(".cu") else ["-x", "c++"]) + extra
        cmd = [cc, *flags, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = OUT / (LIB.name + ".tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_oracle() -> Path:
    """Compile the CPU oracle (test infrastructure) with its Makefile."""
    r = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return ROOT / "oracle" / "_build" / "liboracle.so"


if __name__ == "__main__":
    print(build(force=True, verbose=True))
