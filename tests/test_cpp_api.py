"""The C++ drop-in classes (include/cudaraster/CudaRaster.hpp): they compile
with the host compiler alone and link against the library (CPU), and a
program written against them draws the cube and a soup bit-exact to the
oracle (GPU)."""
import subprocess

import numpy as np
import pytest

from conftest import pkg_mod
from cpp_build import build_draw_file
from helpers import PIPE_SAMPLES, assert_same, oracle_render, pkg, vertices_for


def test_header_compiles_and_links(tmp_path):
    exe = build_draw_file(tmp_path)
    assert exe.exists()


def _write_scene(path, pipe, sc, clear_rgba, clear_depth):
    verts = vertices_for(pipe, sc["vertices"])
    idx = np.ascontiguousarray(sc["indices"], dtype=np.int32)
    name = pipe.encode().ljust(64, b"\0")
    with open(path, "wb") as f:
        np.array([sc["width"], sc["height"], PIPE_SAMPLES.get(pipe, 1), verts.shape[0], verts.shape[1] * 4,
                  idx.shape[0], 1], np.int32).tofile(f)
        np.array(list(clear_rgba) + [clear_depth], np.float32).tofile(f)
        f.write(name)
        verts.tofile(f)
        idx.tofile(f)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cube", "soup_srcover_msaa4"])
def test_cpp_program_matches_oracle(cuda, tmp_path, case):
    scenes = pkg_mod("scenes")
    if case == "cube":
        pipe, sc = "PixelPipe_gouraud", scenes.cube()
    else:
        pipe = "PixelPipe_gouraud_srcover_msaa4"
        sc = scenes.soup(20000, 640, 360, seed=31, median_px=6.0, alpha_range=(0.2, 1.0))
    rgba, zc = (0.2, 0.4, 0.8, 1.0), 1.0
    _write_scene(tmp_path / "scene.bin", pipe, sc, rgba, zc)
    exe = build_draw_file(tmp_path)
    res = subprocess.run([str(exe), str(tmp_path / "scene.bin"), str(tmp_path / "out.bin")], capture_output=True,
                         text=True)
    assert res.returncode == 0, res.stderr
    assert "setup" in res.stdout
    p = pkg()
    clear = (p.color_to_abgr(*rgba), p.clear_depth_from_float(zc))
    rc, rd, st = oracle_render(pipe, sc, clear)
    out = np.fromfile(tmp_path / "out.bin", dtype=np.uint32)
    gc, gd = out[:rc.size].reshape(rc.shape), out[rc.size:].reshape(rd.shape)
    assert_same(gc, gd, rc, rd, f"C++ API {case}")
