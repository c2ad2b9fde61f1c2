"""In-tree build of the native library ``glslppm_gb300/_lib/libsppm.so``.

Host C++ (scene ingest, BVH build) is compiled with g++; the CUDA translation units with nvcc for
sm_103a only (``-gencode arch=compute_103a,code=sm_103a``).  Every translation unit is compiled with
``-ffp-contract=off`` on the host side; the plain-FP32 kernels additionally with ``-fmad=false``.
Translation units compile in parallel; a unit is rebuilt when it or a header it includes changed.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
OBJ_DIR = PKG / "_build"
LIB_DIR = PKG / "_lib"
LIB = LIB_DIR / "libsppm.so"
INCLUDE = REPO / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (set NVCC or put CUDA's bin directory on PATH)")


def _units() -> list[tuple[Path, list[str]]]:
    nvcc = _nvcc()
    inc = [f"-I{INCLUDE}", f"-I{CSRC}"]
    units = []
    for src in sorted((CSRC / "host").glob("*.cpp")):
        units.append((src, ["g++", "-std=c++17", *HOST_FLAGS, "-Wall", *inc, "-c", str(src)]))
    for src in sorted((CSRC / "cuda").glob("*.cu")):
        extra = ["-fmad=false"] if src.name.endswith("_fp32.cu") else []
        units.append((src, [nvcc, "-std=c++17", "-O3", *ARCH, "-lineinfo", *extra,
                            "-Xcompiler", ",".join(HOST_FLAGS), *inc, "-c", str(src)]))
    return units


def _headers() -> list[Path]:
    return [*INCLUDE.glob("*.h"), *CSRC.rglob("*.h"), *CSRC.rglob("*.cuh")]


def _compile(unit: tuple[Path, list[str]], newest_header: float, force: bool) -> Path:
    src, cmd = unit
    obj = OBJ_DIR / (src.parent.name + "_" + src.name + ".o")
    if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, newest_header):
        tmp = obj.with_suffix(f".o.tmp{os.getpid()}")
        proc = subprocess.run([*cmd, "-o", str(tmp)], capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"compiling {src.name} failed:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
        os.replace(tmp, obj)
    return obj


def build(force: bool = False, jobs: int | None = None) -> Path:
    """Compile and link libsppm.so; returns its path."""
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    units = _units()
    newest = max(h.stat().st_mtime for h in _headers())
    with ThreadPoolExecutor(max_workers=jobs or min(len(units), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda u: _compile(u, newest, force), units))
    if force or not LIB.exists() or LIB.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
        cmd = [_nvcc(), "-shared", *ARCH, *map(str, objs), "-o", str(tmp), "-lpthread"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"linking libsppm.so failed:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
