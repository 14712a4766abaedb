"""Host API error paths through the C ABI (a context needs a GPU): invalid
tuning values, drawing before the state is complete and a pipe whose sample
count differs from the surfaces' are rejected with a status and a message,
and the context stays usable afterwards."""
import numpy as np
import pytest
import torch

from conftest import pkg_mod
from helpers import assert_same, gpu_render, oracle_render, pkg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bad,words", [(dict(bin_log2=6), "bin_log2"), (dict(bin_log2=2), "bin_log2"),
                                       (dict(fine_warps=3), "fine_warps"), (dict(fine_warps=16), "fine_warps"),
                                       (dict(bin_chunk_tris=33), "bin_chunk_tris"),
                                       (dict(fine_self_pixels=65), "fine_self_pixels"),
                                       (dict(fine_self_pixels=-1), "fine_self_pixels")])
def test_invalid_tuning_rejected(cuda, bad, words):
    p = pkg()
    cr = p.CudaRaster()
    cr.init()
    with pytest.raises(p.RasterError, match=words):
        cr.setTuning(**bad)


def test_draw_needs_state_and_matching_samples(cuda):
    p = pkg()
    cr = p.CudaRaster()
    cr.init()
    with pytest.raises(p.RasterError, match="Surfaces not set"):
        cr.drawTriangles()
    color = p.CudaSurface((64, 64), p.CudaSurface.FORMAT_RGBA8, 4)
    depth = p.CudaSurface((64, 64), p.CudaSurface.FORMAT_DEPTH32, 4)
    cr.setSurfaces(color, depth)
    with pytest.raises(p.RasterError, match="Pixel pipe not set"):
        cr.drawTriangles()
    cr.setPixelPipe(None, "PixelPipe_gouraud")   # one sample per pixel
    v = torch.zeros((3, 8), dtype=torch.float32, device="cuda")
    i = torch.arange(3, dtype=torch.int32, device="cuda")
    cr.setVertexBuffer(v, 0)
    cr.setIndexBuffer(i, 0, 1)
    with pytest.raises(p.RasterError, match="Mismatch in multisampling"):
        cr.drawTriangles()


def test_context_usable_after_errors(cuda):
    p = pkg()
    scenes = pkg_mod("scenes")
    sc = scenes.soup(2000, 200, 150, seed=41, median_px=6.0)
    clear = (p.color_to_abgr(0.1, 0.2, 0.3, 1.0), p.clear_depth_from_float(1.0))
    cr = p.CudaRaster()
    cr.init()
    with pytest.raises(p.RasterError):
        cr.setTuning(bin_log2=9)
    gc, gd, _, _ = gpu_render("PixelPipe_gouraud", sc, clear, cr=cr)
    rc, rd, _ = oracle_render("PixelPipe_gouraud", sc, clear)
    assert_same(gc, gd, rc, rd, "after rejected tuning")
