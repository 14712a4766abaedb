"""Cell grids at their limits, against the CPU oracle: a 4000x1000 viewport
with 64-px bins (63 x 16 = 1008 bins, bounding boxes up to 63 bins wide) and
with 256-px bins (32 x 32 tiles per bin), drawn with a mix of small triangles
and triangles hundreds of pixels across -- items with more (item, cell)
pairs than a warp has lanes in the bin, coarse and fine stages, on both sides
of the fine stage's self-rasterization threshold."""
import numpy as np
import pytest

from conftest import pkg_mod
from helpers import assert_same, gpu_render, oracle_render, pkg

pytestmark = pytest.mark.gpu

W, H = 4000, 1000


def _scene(alpha: bool):
    scenes = pkg_mod("scenes")
    ar = (0.2, 1.0) if alpha else None
    small = scenes.soup(4000, W, H, seed=31, median_px=5.0, alpha_range=ar)
    large = scenes.soup(60, W, H, seed=32, median_px=500.0, sigma=0.6, alpha_range=ar)
    verts = np.concatenate([small["vertices"], large["vertices"]])
    # Large triangles interleaved with the small ones, so every batch mixes sizes.
    idx_s, idx_l = small["indices"], large["indices"] + small["vertices"].shape[0]
    order = np.concatenate([idx_s[:2000], idx_l[:30], idx_s[2000:], idx_l[30:]])
    return {"vertices": verts, "indices": np.ascontiguousarray(order, dtype=np.int32), "width": W, "height": H}


@pytest.mark.parametrize("pipe", ["PixelPipe_gouraud", "PixelPipe_gouraud_srcover", "PixelPipe_gouraud_msaa4"])
@pytest.mark.parametrize("tuning", [dict(bin_log2=3), dict(bin_log2=3, fine_self_pixels=64),
                                    dict(bin_log2=5, fine_self_pixels=2)])
def test_wide_grids_match_oracle(cuda, pipe, tuning):
    p = pkg()
    sc = _scene("srcover" in pipe)
    clear = (p.color_to_abgr(0.1, 0.2, 0.3, 1.0), p.clear_depth_from_float(1.0))
    rc, rd, st = oracle_render(pipe, sc, clear)
    assert st["zmin_violations"] == 0
    gc, gd, counters, _ = gpu_render(pipe, sc, clear, tuning=tuning)
    assert counters["overflow"] == 0
    assert counters["num_bins"] == (1008 if tuning["bin_log2"] == 3 else 64)
    assert_same(gc, gd, rc, rd, f"{pipe} {tuning}")
