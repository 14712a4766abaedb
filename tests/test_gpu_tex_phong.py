"""The textured Phong pipe (the reference's PixelPipe_texPhong, test/shader/
Shaders.cu:117-199) against the CPU oracle: the atlas filter bit for bit, the
filter against the GPU's texture unit within its weight precision, and whole
frames -- vertex shader, per-fragment lighting, two mip lookups, alpha test --
bit for bit at 1 spp, in quad mode, with 4x MSAA and blended over existing
content."""
import numpy as np
import pytest
import torch

from conftest import pkg_mod
from helpers import assert_same, gpu_render, init_surfaces, oracle_render, pkg
from oracle import oracle as orc
from oracle import vertex_oracle as vo

pytestmark = pytest.mark.gpu


def _uv(n, seed):
    rng = np.random.default_rng(seed)
    uv = rng.uniform(-3.0, 3.0, (n, 2)).astype(np.float32)
    uv[: n // 4] = rng.uniform(0.0, 1.0, (n // 4, 2))
    # Texel centres, half-way points, exact integers and non-finite values.
    uv[-8:] = [[0.5 / 256, 0.5 / 128], [1.0 / 256, 1.0 / 128], [0.0, 0.0], [1.0, -1.0],
               [np.nan, 0.25], [np.inf, -np.inf], [-1e-9, 1e-9], [7.999999, -7.999999]]
    return uv


def _atlas(seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 2**32, (128, 256), dtype=np.uint64).astype(np.uint32)


def test_texture_filter_bit_exact(cuda):
    raster = pkg_mod("raster")
    atlas = _atlas(1)
    uv = _uv(100_000, 2)
    got = raster.texture_sample(torch.from_numpy(atlas.view(np.int32)).cuda(), torch.from_numpy(uv).cuda()).cpu().numpy()
    ref = orc.texture_sample(atlas, uv)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_texture_filter_matches_texture_unit(cuda):
    # The specified filter rounds the 8-bit weights to nearest; the texture unit's
    # filter quantizes them to 8 fractional bits as well, so the two agree to within
    # one weight step per axis (2/256 of the texel range) and on average far closer.
    raster = pkg_mod("raster")
    atlas = _atlas(3)
    uv = _uv(100_000, 4)[:-8]
    a = torch.from_numpy(atlas.view(np.int32)).cuda()
    u = torch.from_numpy(uv).cuda()
    sw = raster.texture_sample(a, u).cpu().numpy()
    hw = raster.texture_sample(a, u, hardware=True).cpu().numpy()
    diff = np.abs(sw - hw)
    assert diff.max() <= 2.0 / 256 + 1e-6, diff.max()
    assert diff.mean() < 2e-3, diff.mean()
    # At texel centres both return the texel itself.
    centres = np.stack(np.meshgrid((np.arange(256) + 0.5) / 256, (np.arange(128) + 0.5) / 128), -1).reshape(-1, 2)
    c = torch.from_numpy(centres.astype(np.float32)).cuda()
    assert np.array_equal(raster.texture_sample(a, c).cpu().numpy(), raster.texture_sample(a, c, hardware=True).cpu().numpy())


def _draw(pipe, sc, clear, color=None, depth=None):
    raster = pkg_mod("raster")
    k = [sc["pos_to_clip"], sc["pos_to_camera"], sc["normal_to_camera"]]
    shaded = raster.vertex_shader_tex_phong(torch.from_numpy(sc["input"]).cuda(), *k).cpu().numpy()
    assert np.array_equal(shaded.view(np.uint32), vo.vertex_tex_phong(sc["input"], *k).view(np.uint32))
    mats = torch.from_numpy(sc["materials"]).cuda()
    tri = torch.from_numpy(sc["triangle_material_idx"]).cuda()
    atlas = torch.from_numpy(sc["atlas"].view(np.int32)).cuda()
    raster.set_tex_phong_constants(mats, tri, atlas)
    orc.set_tex_phong(sc["materials"], sc["triangle_material_idx"], sc["atlas"])
    scene = {"vertices": shaded, "indices": sc["indices"], "width": sc["width"], "height": sc["height"]}
    gc, gd, _, _ = gpu_render(pipe, scene, clear, color, depth)
    rc, rd, st = oracle_render(pipe, scene, clear, color, depth)
    assert st["zmin_violations"] == 0
    return gc, gd, rc, rd


@pytest.mark.parametrize("pipe", ["PixelPipe_texPhong", "PixelPipe_texPhong_quads", "PixelPipe_texPhong_msaa4"])
def test_textured_terrain_bit_exact(cuda, pipe):
    p = pkg()
    scenes = pkg_mod("scenes")
    sc = scenes.textured_terrain(128, 640, 480, seed=5)
    clear = (p.color_to_abgr(0.1, 0.2, 0.3, 1.0), p.clear_depth_from_float(1.0))
    gc, gd, rc, rd = _draw(pipe, sc, clear)
    bg = int((rc == clear[0]).sum())
    assert bg < rc.size * 0.8, "terrain not drawn"
    assert_same(gc, gd, rc, rd, pipe)


def test_textured_terrain_srcover_over_content(cuda):
    scenes = pkg_mod("scenes")
    sc = scenes.textured_terrain(96, 512, 384, seed=6, frame=40.0)
    color, depth = init_surfaces(sc, 1, seed=7)
    depth[:] = np.maximum(depth, np.uint32(0x80000000))   # leave room in front of the old content
    gc, gd, rc, rd = _draw("PixelPipe_texPhong_srcover", sc, None, color, depth)
    assert_same(gc, gd, rc, rd, "texPhong srcover")


def test_alpha_test_discards(cuda):
    # Only the alpha-textured material: its holes leave the clear colour and depth.
    p = pkg()
    scenes = pkg_mod("scenes")
    sc = scenes.textured_terrain(64, 320, 240, seed=8)
    sc["triangle_material_idx"] = np.full_like(sc["triangle_material_idx"], 2)
    clear = (p.color_to_abgr(0.0, 0.0, 0.0, 1.0), p.clear_depth_from_float(1.0))
    gc, gd, rc, rd = _draw("PixelPipe_texPhong", sc, clear)
    assert_same(gc, gd, rc, rd, "alpha test")
    assert int((rc == clear[0]).sum()) > 0


def test_tex_phong_constants_validation(cuda):
    lib = pkg_mod("_lib").load()
    m = torch.zeros((1, 144), dtype=torch.float32, device="cuda")
    t = torch.zeros(4, dtype=torch.int32, device="cuda")
    a = torch.zeros((2, 2), dtype=torch.int32, device="cuda")
    ok = lib.cr_set_tex_phong_constants(m.data_ptr(), 1, t.data_ptr(), 4, a.data_ptr(), 2, 2, None)
    assert ok == 0
    bad = [(0, 1, t.data_ptr(), 4, a.data_ptr(), 2, 2), (m.data_ptr(), 0, t.data_ptr(), 4, a.data_ptr(), 2, 2),
           (m.data_ptr(), 1, None, 4, a.data_ptr(), 2, 2), (m.data_ptr(), 1, t.data_ptr(), 0, a.data_ptr(), 2, 2),
           (m.data_ptr(), 1, t.data_ptr(), 4, None, 2, 2), (m.data_ptr(), 1, t.data_ptr(), 4, a.data_ptr(), 0, 2)]
    for args in bad:
        assert lib.cr_set_tex_phong_constants(*args, None) == 1


@pytest.mark.parametrize("tuning", [dict(bin_log2=3, fine_warps=4), dict(bin_log2=5, bin_chunk_tris=96),
                                    dict(fine_self_pixels=1, coarse_unit_entries=64),
                                    dict(fine_self_pixels=64, fine_warps=8)])
def test_textured_tuning_invariance(cuda, tuning):
    # Tuning changes queues and work distribution, never a bit of the textured frame.
    p = pkg()
    raster = pkg_mod("raster")
    scenes = pkg_mod("scenes")
    sc = scenes.textured_terrain(96, 512, 384, seed=13)
    k = [sc["pos_to_clip"], sc["pos_to_camera"], sc["normal_to_camera"]]
    shaded = raster.vertex_shader_tex_phong(torch.from_numpy(sc["input"]).cuda(), *k).cpu().numpy()
    raster.set_tex_phong_constants(torch.from_numpy(sc["materials"]).cuda(),
                                   torch.from_numpy(sc["triangle_material_idx"]).cuda(),
                                   torch.from_numpy(sc["atlas"].view(np.int32)).cuda())
    scene = {"vertices": shaded, "indices": sc["indices"], "width": 512, "height": 384}
    clear = (p.color_to_abgr(0.1, 0.2, 0.3, 1.0), p.clear_depth_from_float(1.0))
    base = gpu_render("PixelPipe_texPhong", scene, clear)
    tuned = gpu_render("PixelPipe_texPhong", scene, clear, tuning=tuning)
    assert_same(tuned[0], tuned[1], base[0], base[1], f"tuning {tuning}")
