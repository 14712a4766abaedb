"""Targeted parity cases for the fine stage's visibility path and the binning
rule at one sample per pixel, against the oracle (FineRaster.inl:244-305 for
coverage, CudaRaster.cpp:669-1403 for the sequential order the results must
match):

* many small triangles per tile: each batch's (triangle, pixel) pairs take
  several 32-pair passes, so triangles whose pairs straddle a pass boundary
  are found through the carried start;
* triangles of one constant depth, small and large mixed: every sample's
  winner is decided by list position alone, across batches and between the
  pair loop and the large-triangle loop of one batch (with src-over, only
  each pixel's first fragment in list order passes the LESS test, the tie
  the ordered path's batch filter must break by position);
* slivers whose vertex boxes cross a tile or bin edge by less than half a
  pixel: at one sample per pixel those cells hold no pixel centre and are
  left out of the lists (the GPU lists must still equal the oracle's rule and
  the frame the oracle's).
"""
import math

import numpy as np
import pytest

from conftest import pkg_mod
from helpers import assert_same, gpu_render, oracle_render, pkg
from test_gpu_queues import _check_level, _gpu_queues
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _records(clip: np.ndarray, rgba: np.ndarray) -> np.ndarray:
    """GouraudVertex records: clip position, then RGBA (32 bytes)."""
    return np.ascontiguousarray(np.concatenate([clip, rgba], axis=1), dtype=np.float32)


def _triangles(centers_px, radii_px, width, height, rng, depth_ndc=None):
    """Triangles around pixel-space centres with the given circumradii, random
    orientation and winding kept front-facing; depth per triangle random in
    NDC unless depth_ndc is given; w random in [1, 4]."""
    n = len(centers_px)
    theta = rng.uniform(0.0, 2.0 * math.pi, n)
    k = np.arange(3)[None, :]
    ang = theta[:, None] + (2.0 * math.pi / 3.0) * k + rng.uniform(-0.3, 0.3, (n, 3))
    px = centers_px[:, 0:1] + radii_px[:, None] * np.cos(ang)
    py = centers_px[:, 1:2] + radii_px[:, None] * np.sin(ang)
    # Counter-clockwise in NDC with y up is front-facing here; fix the winding per triangle.
    area = (px[:, 1] - px[:, 0]) * (py[:, 2] - py[:, 0]) - (px[:, 2] - px[:, 0]) * (py[:, 1] - py[:, 0])
    flip = area < 0
    px[flip] = px[flip][:, ::-1]
    py[flip] = py[flip][:, ::-1]
    nx = px * (2.0 / width) - 1.0
    ny = py * (2.0 / height) - 1.0
    z = rng.uniform(-0.9, 0.9, n) if depth_ndc is None else np.full(n, depth_ndc)
    w = rng.uniform(1.0, 4.0, n)
    clip = np.stack([nx * w[:, None], ny * w[:, None], (z * w)[:, None].repeat(3, 1), w[:, None].repeat(3, 1)],
                    axis=-1).reshape(-1, 4)
    rgba = rng.integers(0, 256, (3 * n, 4)).astype(np.float32) / np.float32(255.0)
    return clip.astype(np.float32), rgba


def _scene(clip, rgba, width, height):
    n = clip.shape[0] // 3
    return {"vertices": _records(clip, rgba), "indices": np.arange(3 * n, dtype=np.int32).reshape(-1, 3),
            "width": width, "height": height}


def _parity(pipe, sc, what):
    p = pkg()
    clear = (p.color_to_abgr(0.1, 0.2, 0.3, 1.0), p.clear_depth_from_float(1.0))
    gc, gd, cnt, _ = gpu_render(pipe, sc, clear)
    rc, rd, _ = oracle_render(pipe, sc, clear)
    assert_same(gc, gd, rc, rd, what)
    return cnt


@pytest.mark.parametrize("pipe", ["PixelPipe_gouraud", "PixelPipe_gouraud_msaa4", "PixelPipe_gouraud_srcover",
                                  "PixelPipe_gouraud_additive"])
def test_many_small_triangles_per_tile(cuda, pipe):
    rng = np.random.default_rng(71)
    W = H = 64
    n = 4000
    centers = rng.uniform(0.0, 64.0, (n, 2))
    radii = rng.uniform(1.0, 2.4, n)            # pixel boxes of about 2x2 to 4x4: all on the pair path
    sc = _scene(*_triangles(centers, radii, W, H, rng), W, H)
    cnt = _parity(pipe, sc, f"{pipe} small triangles")
    # About a hundred entries per tile: several batches, each with many 32-pair passes.
    assert cnt["tile_entries"] > 60 * cnt["num_tiles"]


@pytest.mark.parametrize("pipe", ["PixelPipe_gouraud", "PixelPipe_gouraud_msaa4", "PixelPipe_gouraud_srcover"])
def test_constant_depth_mixed_sizes_keep_list_order(cuda, pipe):
    rng = np.random.default_rng(72)
    W = H = 96
    n = 1500
    centers = rng.uniform(0.0, 96.0, (n, 2))
    radii = np.exp(rng.normal(math.log(3.0), 1.0, n))   # small (pair loop) and large (warp-wide) triangles
    sc = _scene(*_triangles(centers, radii, W, H, rng, depth_ndc=0.25), W, H)
    _parity(pipe, sc, f"{pipe} constant depth")


def test_slivers_at_cell_edges(cuda):
    rng = np.random.default_rng(73)
    W, H = 256, 192
    n = 3000
    # Centres on tile edges (multiples of 8 px) in x or y; boxes cross the edge by
    # 0.05-0.45 px on one side and extend a few pixels on the other.
    edge_x = rng.integers(1, W // 8, n) * 8.0
    edge_y = rng.integers(1, H // 8, n) * 8.0
    vertical = rng.uniform(0.0, 1.0, n) < 0.5
    lo = rng.uniform(0.05, 0.45, n)
    hi = rng.uniform(1.5, 5.0, n)
    along = rng.uniform(4.0, float(min(W, H)) - 4.0, n)
    span = rng.uniform(1.5, 6.0, n)
    side = np.where(rng.uniform(0.0, 1.0, n) < 0.5, 1.0, -1.0)
    a0 = np.where(vertical, edge_x - side * lo, along)
    b0 = np.where(vertical, along, edge_y - side * lo)
    x = np.stack([a0, np.where(vertical, edge_x + side * hi, along + span), np.where(vertical, edge_x + side * hi, along)], 1)
    y = np.stack([b0, np.where(vertical, along, edge_y + side * hi), np.where(vertical, along + span, edge_y + side * hi)], 1)
    area = (x[:, 1] - x[:, 0]) * (y[:, 2] - y[:, 0]) - (x[:, 2] - x[:, 0]) * (y[:, 1] - y[:, 0])
    flip = area < 0
    x[flip] = x[flip][:, ::-1]
    y[flip] = y[flip][:, ::-1]
    nx, ny = x * (2.0 / W) - 1.0, y * (2.0 / H) - 1.0
    z = rng.uniform(-0.9, 0.9, n)
    clip = np.stack([nx, ny, np.repeat(z[:, None], 3, 1), np.ones_like(nx)], -1).reshape(-1, 4).astype(np.float32)
    rgba = rng.integers(0, 256, (3 * n, 4)).astype(np.float32) / np.float32(255.0)
    sc = _scene(clip, rgba, W, H)
    _parity("PixelPipe_gouraud", sc, "slivers")
    # Queue lists: equal to the oracle's rule at every bin size, which at one
    # sample leaves out the cells the slivers only graze.
    p = pkg()
    lib = pkg_mod("_lib").load()
    op = orc.make_pipe(W, H, 1, orc.DEPTH | orc.LERP, "replace", "gouraud", 32)
    for bin_log2 in (3, 4):
        cr = p.CudaRaster()
        cr.init()
        cr.setTuning(bin_log2=bin_log2)
        gpu_render("PixelPipe_gouraud", sc, None, cr=cr)
        bins, tiles = _gpu_queues(cr, lib)
        q = {k: orc.queue_lists(op, sc["vertices"], sc["indices"], bin_log2, k) for k in orc.QUEUE_KINDS}
        what = f"slivers, bins of {8 << bin_log2} px"
        _check_level("bin", bins, q["bin_exact"], q["bin_rule"], what)
        _, n_tile = _check_level("tile", tiles, q["tile_exact"], q["tile_rule"], what)
        # The vertex boxes would have put every sliver in the tiles on both sides of its edge.
        assert n_tile < 2 * n
