"""Build recipe for the native library (and the CPU oracle used by the tests).

Compiles every .cu file of csrc/ for sm_103a in parallel with nvcc and links
them into libcudaraster_gb300.so next to this file. No cmake, no torch
extension machinery: the library is a plain C-ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
INCLUDE = REPO_DIR / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "libcudaraster_gb300.so"
LIB_PATH = PKG_DIR / LIB_NAME

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH_FLAGS + [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
    f"-I{INCLUDE}", f"-I{CSRC}",
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the rasterizer")
    return cand


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.rglob("*.h"))
                  + list(INCLUDE.rglob("*.hpp")) + list(INCLUDE.rglob("*.cuh")) + list(INCLUDE.rglob("*.inl")))


def _compile(src: Path, extra: list[str]) -> Path:
    obj = BUILD_DIR / (src.stem + ".o")
    cmd = [nvcc(), *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj


def build_library(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile csrc/*.cu into LIB_PATH (incremental on source timestamps)."""
    extra = list(extra or [])
    newest = max(p.stat().st_mtime for p in _deps())
    if not force and LIB_PATH.exists() and LIB_PATH.stat().st_mtime >= newest and not extra:
        return LIB_PATH
    BUILD_DIR.mkdir(exist_ok=True)
    srcs = _sources()
    workers = min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH_FLAGS, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    if verbose:
        print(f"built {LIB_PATH}")
    return LIB_PATH


def reference_dir() -> Path | None:
    """The reference sources (tcoppex/cudaraster-linux checkout) named by the
    CR_REFERENCE_DIR environment variable, if it is set and holds them."""
    d = os.environ.get("CR_REFERENCE_DIR")
    if not d:
        return None
    p = Path(d)
    return p if (p / "src" / "cudaraster" / "cuda" / "PixelPipe.inl").exists() else None


def build_oracle(with_reference: bool | None = None) -> None:
    """Build oracle/liboracle.so, and oracle/_ref when CR_REFERENCE_DIR names the
    reference sources."""
    oracle_dir = REPO_DIR / "oracle"
    res = subprocess.run(["make", "-C", str(oracle_dir), "liboracle.so"], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    ref = reference_dir()
    if with_reference is None:
        with_reference = ref is not None
    if with_reference:
        if ref is None:
            raise RuntimeError("set CR_REFERENCE_DIR to the reference sources to build oracle/_ref")
        res = subprocess.run(["make", "-C", str(oracle_dir), "ref", f"REF={ref}"], capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"reference harness build failed:\n{res.stdout}\n{res.stderr}")


if __name__ == "__main__":
    build_library(force="--force" in sys.argv, verbose=True)
    build_oracle()
