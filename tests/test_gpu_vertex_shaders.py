"""The Gouraud-lighting and texPhong vertex shaders and their exact power on
the GPU, bit for bit against the CPU oracle, and the lit vertices drawn
through the rasterizer against the CPU oracle's render."""
import numpy as np
import pytest
import torch

from conftest import pkg_mod
from helpers import assert_same, gpu_render, oracle_render, pkg
from oracle import vertex_oracle as vo

pytestmark = pytest.mark.gpu


def _camera():
    scenes = pkg_mod("scenes")
    view = scenes.look_at((1.5, 2.0, 3.0), (0.0, 0.0, 0.0)).astype(np.float32)
    proj = scenes.perspective(60.0, 4.0 / 3.0, 0.1, 100.0).astype(np.float32)
    clip = (proj @ view).astype(np.float32)
    normal = view[:3, :3].copy()
    return clip, view, normal


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    v = np.zeros((n, 8), np.float32)
    v[:, 0:3] = rng.uniform(-1.5, 1.5, (n, 3))
    nrm = rng.normal(size=(n, 3))
    nrm[::97] = 0.0                      # zero normals
    v[:, 3:6] = nrm
    v[:, 6:8] = rng.uniform(0, 1, (n, 2))
    v[::89, 0:3] = 0.0                   # positions at the model origin
    mats = np.zeros((7, 8), np.float32)
    mats[:, 0:4] = rng.uniform(0, 1, (7, 4))
    mats[:, 4:7] = rng.uniform(0, 1, (7, 3))
    mats[:, 7] = rng.uniform(0.5, 128, 7)
    idx = rng.integers(-2, 9, n).astype(np.int32)   # out of range clamps to the table
    return v, mats, idx


def test_pow_exact_bit_exact(cuda):
    raster = pkg_mod("raster")
    rng = np.random.default_rng(5)
    x = np.concatenate([rng.uniform(0, 1, 50_000), rng.uniform(0, 4, 10_000), [0, 0, 1e-45, 1e-40, np.inf, 1]])
    y = np.concatenate([rng.uniform(0.25, 128, 50_000), rng.uniform(-8, 8, 10_000), [2, 0, 1, 3, 2, -1]])
    x, y = x.astype(np.float32), y.astype(np.float32)
    got = raster.pow_exact(torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()).cpu().numpy()
    ref = vo.pow_exact(x, y)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_gouraud_vertex_shader_bit_exact(cuda):
    raster = pkg_mod("raster")
    clip, view, normal = _camera()
    v, mats, idx = _inputs(100_000, 6)
    got = raster.vertex_shader_gouraud(torch.from_numpy(v).cuda(), clip, view, normal, torch.from_numpy(mats).cuda(),
                                       torch.from_numpy(idx).cuda()).cpu().numpy()
    ref = vo.vertex_gouraud(v, clip, view, normal, mats, idx)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_tex_phong_vertex_shader_bit_exact(cuda):
    raster = pkg_mod("raster")
    clip, view, normal = _camera()
    v, _, _ = _inputs(50_000, 7)
    got = raster.vertex_shader_tex_phong(torch.from_numpy(v).cuda(), clip, view, normal).cpu().numpy()
    ref = vo.vertex_tex_phong(v, clip, view, normal)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_lit_mesh_renders_as_oracle(cuda):
    # The heightfield, lit per vertex on the GPU, drawn by the Gouraud pipe.
    p = pkg()
    raster = pkg_mod("raster")
    scenes = pkg_mod("scenes")
    pos, _, idx = scenes.grid_mesh(96, seed=9)
    n = pos.shape[0]
    rng = np.random.default_rng(10)
    v = np.zeros((n, 8), np.float32)
    v[:, 0:3] = pos
    v[:, 3:6] = np.array([0, 1, 0], np.float32) + rng.normal(scale=0.2, size=(n, 3)).astype(np.float32)
    mats = np.array([[0.7, 0.6, 0.3, 1.0, 0.4, 0.4, 0.4, 24.0], [0.2, 0.5, 0.8, 1.0, 0.9, 0.9, 0.9, 64.0]], np.float32)
    midx = (np.arange(n) % 2).astype(np.int32)
    clip, view, normal = _camera()
    lit = raster.vertex_shader_gouraud(torch.from_numpy(v).cuda(), clip, view, normal, torch.from_numpy(mats).cuda(),
                                       torch.from_numpy(midx).cuda()).cpu().numpy()
    assert np.array_equal(lit.view(np.uint32), vo.vertex_gouraud(v, clip, view, normal, mats, midx).view(np.uint32))
    sc = {"vertices": lit, "indices": np.ascontiguousarray(idx, dtype=np.int32), "width": 640, "height": 480}
    clear = (p.color_to_abgr(0.0, 0.0, 0.0, 1.0), p.clear_depth_from_float(1.0))
    gc, gd, _, _ = gpu_render("PixelPipe_gouraud", sc, clear)
    rc, rd, st = oracle_render("PixelPipe_gouraud", sc, clear)
    assert st["zmin_violations"] == 0
    assert_same(gc, gd, rc, rd, "lit heightfield")


def test_vertex_shaders_unaligned_records(cuda):
    # texPhong records only 4-byte aligned take the per-thread path, 16-byte aligned
    # ones are staged through shared memory; both give the oracle's bits, also for a
    # vertex count that leaves the last block partly empty (Gouraud takes the
    # per-thread path either way).
    raster = pkg_mod("raster")
    clip, view, normal = _camera()
    v, mats, idx = _inputs(10_007, 8)
    flat = torch.zeros(v.size + 1, dtype=torch.float32, device="cuda")
    flat[1:] = torch.from_numpy(v.reshape(-1)).cuda()
    shifted = flat[1:].view(v.shape)
    assert shifted.data_ptr() % 16 == 4
    aligned = torch.from_numpy(v).cuda()
    m = torch.from_numpy(mats).cuda()
    i = torch.from_numpy(idx).cuda()
    ref_g = vo.vertex_gouraud(v, clip, view, normal, mats, idx).view(np.uint32)
    ref_t = vo.vertex_tex_phong(v, clip, view, normal).view(np.uint32)
    for src in (shifted, aligned):
        g = raster.vertex_shader_gouraud(src, clip, view, normal, m, i).cpu().numpy()
        t = raster.vertex_shader_tex_phong(src, clip, view, normal).cpu().numpy()
        assert np.array_equal(g.view(np.uint32), ref_g)
        assert np.array_equal(t.view(np.uint32), ref_t)
