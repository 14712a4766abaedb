"""Builds tests/cpp/draw_file.cpp with the host C++ compiler against the C++
drop-in header and the rasterizer library (used by the C++ API tests)."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
LIB_DIR = ROOT / "cudaraster-linux_gb300"


def cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parents[1]
    return Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def build_draw_file(out_dir: Path) -> Path:
    cuda = cuda_home()
    exe = out_dir / "draw_file"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", f"-I{ROOT / 'include'}", f"-I{cuda / 'include'}",
           str(ROOT / "tests" / "cpp" / "draw_file.cpp"), "-o", str(exe), f"-L{LIB_DIR}", "-lcudaraster_gb300",
           f"-Wl,-rpath,{LIB_DIR}", f"-L{cuda / 'lib64'}", "-lcudart", f"-Wl,-rpath,{cuda / 'lib64'}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"C++ build failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if res.stderr.strip():
        raise RuntimeError(f"C++ build warnings:\n{res.stderr}")
    return exe
