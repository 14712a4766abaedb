"""Batched drawing, captured graphs, tuning invariance and the overflow rerun
path: every framebuffer must be bit-identical to a plain single-scene draw
and to the CPU oracle."""
import numpy as np
import pytest
import torch

from conftest import pkg_mod
from helpers import PIPE_SAMPLES, assert_same, gpu_render, oracle_render, pkg, vertices_for

pytestmark = pytest.mark.gpu


def _clear():
    p = pkg()
    return (p.color_to_abgr(0.1, 0.2, 0.3, 1.0), p.clear_depth_from_float(1.0))


def _batch_scenes():
    scenes = pkg_mod("scenes")
    specs = [("PixelPipe_gouraud", 3000, (256, 256)), ("PixelPipe_gouraud_srcover", 1500, (300, 200)),
             ("PixelPipe_gouraud", 12000, (512, 512)), ("PixelPipe_gouraud_msaa4", 2000, (160, 120)),
             ("PixelPipe_trihash_srcover", 800, (96, 80)), ("PixelPipe_gouraud_srcover", 5000, (640, 360)),
             ("PixelPipe_gouraud", 1, (64, 64)), ("PixelPipe_gouraud", 7000, (333, 257))]
    out = []
    for k, (pipe, n, (w, h)) in enumerate(specs):
        sc = scenes.soup(n, w, h, seed=100 + k, median_px=5.0,
                         alpha_range=(0.2, 1.0) if "srcover" in pipe else None)
        sc["samples"] = PIPE_SAMPLES.get(pipe, 1)
        out.append((pipe, sc))
    return out


def _instances(items, clear):
    p = pkg()
    insts, keep = [], []
    for pipe, sc in items:
        s = PIPE_SAMPLES.get(pipe, 1)
        cs = p.CudaSurface((sc["width"], sc["height"]), p.CudaSurface.FORMAT_RGBA8, s)
        ds = p.CudaSurface((sc["width"], sc["height"]), p.CudaSurface.FORMAT_DEPTH32, s)
        v = torch.from_numpy(vertices_for(pipe, sc["vertices"])).cuda()
        i = torch.from_numpy(np.ascontiguousarray(sc["indices"], dtype=np.int32)).cuda()
        keep.append((cs, ds, v, i))
        insts.append({"pipe": pipe, "color": cs, "depth": ds, "vertices": v, "indices": i,
                      "numTris": i.shape[0], "clear": clear})
    return insts, keep


def _clear_tuple(clear_words):
    return None


def test_batch_matches_single_draws_and_oracle(cuda):
    items = _batch_scenes()
    p = pkg()
    cr = p.CudaRaster()
    cr.init()
    insts, keep = _instances(items, (0.1, 0.2, 0.3, 1.0, 1.0))
    cr.drawBatch(insts)
    torch.cuda.synchronize()
    clear = _clear()
    for (pipe, sc), (cs, ds, _, _) in zip(items, keep):
        gc = cs.download().numpy().astype(np.uint32)
        gd = ds.download().numpy().astype(np.uint32)
        sc_c, sc_d, _, _ = gpu_render(pipe, sc, clear)
        assert_same(gc, gd, sc_c, sc_d, f"batch vs single {pipe} {sc['width']}x{sc['height']}")
        rc, rd, st = oracle_render(pipe, sc, clear)
        assert st["zmin_violations"] == 0
        assert_same(gc, gd, rc, rd, f"batch vs oracle {pipe}")


def test_batch_graph_replays(cuda):
    items = _batch_scenes()
    p = pkg()
    cr = p.CudaRaster()
    cr.init()
    insts, keep = _instances(items, (0.1, 0.2, 0.3, 1.0, 1.0))
    graph = cr.createBatchGraph(insts)
    clear = _clear()
    refs = [gpu_render(pipe, sc, clear)[:2] for pipe, sc in items]
    for rep in range(3):
        for cs, ds, _, _ in keep:
            cs.tensor.fill_(rep + 1)
            ds.tensor.fill_(rep + 7)
        graph.launch()
        c = graph.counters()
        assert c["overflow"] == 0
        for (rc, rd), (cs, ds, _, _) in zip(refs, keep):
            assert_same(cs.download().numpy().astype(np.uint32), ds.download().numpy().astype(np.uint32), rc, rd,
                        f"graph replay {rep}")
    graph.destroy()


TUNINGS = [dict(bin_log2=3), dict(bin_log2=5), dict(fine_warps=2), dict(fine_warps=4, fine_ctas_per_sm=1),
           dict(fine_self_pixels=1), dict(fine_self_pixels=64),
           dict(bin_chunk_tris=96, coarse_unit_entries=64), dict(bin_chunk_tris=8192, coarse_unit_entries=4096),
           dict(bin_log2=3, fine_warps=8, bin_chunk_tris=1024, coarse_unit_entries=128)]


@pytest.mark.parametrize("pipe", ["PixelPipe_gouraud", "PixelPipe_gouraud_srcover", "PixelPipe_gouraud_msaa4"])
def test_tuning_does_not_change_bits(cuda, pipe):
    sc = pkg_mod("scenes").soup(30000, 700, 500, seed=21, median_px=7.0,
                                alpha_range=(0.2, 1.0) if "srcover" in pipe else None)
    clear = _clear()
    base_c, base_d, _, _ = gpu_render(pipe, sc, clear)
    for t in TUNINGS:
        c, d, _, _ = gpu_render(pipe, sc, clear, tuning=t)
        assert_same(c, d, base_c, base_d, f"{pipe} tuning {t}")


def test_overflow_rerun_is_exact(cuda):
    sc = pkg_mod("scenes").soup(20000, 400, 300, seed=5, median_px=30.0)
    clear = _clear()
    base_c, base_d, _, _ = gpu_render("PixelPipe_gouraud", sc, clear)
    c, d, cnt, _ = gpu_render("PixelPipe_gouraud", sc, clear, capacity=(20001, 1000, 1000))
    assert cnt["reruns"] >= 1 and cnt["overflow"] == 0
    assert_same(c, d, base_c, base_d, "overflow rerun")


def test_batch_with_textured_pipes(cuda):
    # Textured Phong instances (1 and 4 samples, one constant set) batched with
    # Gouraud soups: each framebuffer equals its single draw, bit for bit.
    raster = pkg_mod("raster")
    scenes = pkg_mod("scenes")
    tsc = scenes.textured_terrain(64, 320, 240, seed=12)
    k = [tsc["pos_to_clip"], tsc["pos_to_camera"], tsc["normal_to_camera"]]
    shaded = raster.vertex_shader_tex_phong(torch.from_numpy(tsc["input"]).cuda(), *k).cpu().numpy()
    mats = torch.from_numpy(tsc["materials"]).cuda()
    tri = torch.from_numpy(tsc["triangle_material_idx"]).cuda()
    atlas = torch.from_numpy(tsc["atlas"].view(np.int32)).cuda()
    raster.set_tex_phong_constants(mats, tri, atlas)
    textured = {"vertices": shaded, "indices": tsc["indices"], "width": 320, "height": 240}
    textured4 = dict(textured, width=200, height=150)
    items = [("PixelPipe_gouraud", pkg_mod("scenes").soup(4000, 256, 192, seed=31, median_px=5.0)),
             ("PixelPipe_texPhong", textured),
             ("PixelPipe_texPhong_msaa4", textured4),
             ("PixelPipe_gouraud_srcover", pkg_mod("scenes").soup(2500, 300, 220, seed=32, median_px=5.0,
                                                                   alpha_range=(0.2, 1.0)))]
    p = pkg()
    cr = p.CudaRaster()
    cr.init()
    insts, keep = _instances(items, (0.1, 0.2, 0.3, 1.0, 1.0))
    cr.drawBatch(insts)
    torch.cuda.synchronize()
    for (pipe, sc), (cs, ds, _, _) in zip(items, keep):
        gc = cs.download().numpy().astype(np.uint32)
        gd = ds.download().numpy().astype(np.uint32)
        rc, rd, _, _ = gpu_render(pipe, sc, _clear())
        assert_same(gc, gd, rc, rd, f"batched {pipe}")
        assert (rc != _clear()[0]).any()
