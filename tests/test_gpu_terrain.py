"""Heightfield terrain seen at a grazing angle (the subpixel-stress and
fly-through configurations, at reduced grid sizes): the GPU vertex stage and
the rasterizer at 4K (beyond the reference's 2048-px viewport cap) and with
4x MSAA, bit for bit against the CPU oracle."""
import numpy as np
import pytest
import torch

from conftest import pkg_mod
from helpers import assert_same, gpu_render, oracle_render, pkg
from oracle import vertex_oracle

pytestmark = pytest.mark.gpu


def _clear():
    p = pkg()
    return (p.color_to_abgr(0.05, 0.1, 0.2, 1.0), p.clear_depth_from_float(1.0))


def test_vertex_shader_bit_exact(cuda):
    raster = pkg_mod("raster")
    rng = np.random.default_rng(3)
    model = rng.uniform(-2, 2, (100_000, 3)).astype(np.float32)
    colors = rng.uniform(0, 1, (100_000, 4)).astype(np.float32)
    mvp = pkg_mod("scenes").terrain_camera(17.0, 1920, 1080).astype(np.float32)
    out = raster.vertex_shader_passthrough(torch.from_numpy(model).cuda(), mvp, torch.from_numpy(colors).cuda())
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    ref = vertex_oracle.vertex_passthrough(model, mvp)
    np.testing.assert_array_equal(got[:, :4].view(np.uint32), ref.view(np.uint32))
    np.testing.assert_array_equal(got[:, 4:], colors)
    # A 4-float position stride without colours (16-byte records): the same bits.
    m4 = torch.ones((model.shape[0], 4), dtype=torch.float32, device="cuda")
    m4[:, :3] = torch.from_numpy(model).cuda()
    clip_only = raster.vertex_shader_passthrough(m4[:, :3], mvp).cpu().numpy()
    np.testing.assert_array_equal(clip_only.view(np.uint32), ref.view(np.uint32))


def _terrain(n, w, h, samples, frame):
    scenes = pkg_mod("scenes")
    raster = pkg_mod("raster")
    pos, rgba, tris = scenes.grid_mesh(n, seed=5)
    mvp = scenes.terrain_camera(frame, w, h).astype(np.float32)
    model = pos.astype(np.float32)
    clip_gpu = raster.vertex_shader_passthrough(torch.from_numpy(model).cuda(), mvp,
                                                torch.from_numpy(rgba).cuda()).cpu().numpy()
    clip_ref = vertex_oracle.vertex_passthrough(model, mvp)
    assert (clip_gpu[:, :4].view(np.uint32) == clip_ref.view(np.uint32)).all()
    return {"vertices": clip_gpu, "indices": tris, "width": w, "height": h, "samples": samples}


@pytest.mark.parametrize("frame", [0.0, 40.0])
def test_terrain_msaa4(cuda, frame):
    sc = _terrain(320, 960, 540, 4, frame)
    clear = _clear()
    gc, gd, cnt, _ = gpu_render("PixelPipe_gouraud_msaa4", sc, clear)
    rc, rd, st = oracle_render("PixelPipe_gouraud_msaa4", sc, clear)
    assert st["zmin_violations"] == 0
    assert_same(gc, gd, rc, rd, "terrain 4x MSAA")


def test_terrain_4k(cuda):
    sc = _terrain(512, 3840, 2160, 1, 120.0)
    clear = _clear()
    gc, gd, cnt, _ = gpu_render("PixelPipe_gouraud", sc, clear)
    rc, rd, st = oracle_render("PixelPipe_gouraud", sc, clear)
    assert st["zmin_violations"] == 0
    assert st["num_clipped"] > 0
    assert_same(gc, gd, rc, rd, "terrain 3840x2160")


def test_terrain_4k_msaa4_srcover(cuda):
    sc = _terrain(256, 3840, 2160, 4, 200.0)
    sc["vertices"][:, 7] = 0.5  # half-transparent everywhere
    clear = _clear()
    gc, gd, _, _ = gpu_render("PixelPipe_gouraud_srcover_msaa4", sc, clear)
    rc, rd, st = oracle_render("PixelPipe_gouraud_srcover_msaa4", sc, clear)
    assert_same(gc, gd, rc, rd, "terrain 4K MSAA src-over")
