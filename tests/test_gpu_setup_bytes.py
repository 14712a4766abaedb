"""Per-stage check of the setup stage: the GPU's CRTriangleHeader /
CRTriangleData words and per-triangle subtriangle counts, read back with
cr_read_setup_output, equal the oracle's setup (TriangleSetup.inl) word for
word -- clipped triangles included, whose subtriangles sit in extra slots
found through the triangle's own header on either side."""
import ctypes as C

import numpy as np
import pytest

from conftest import pkg_mod
from helpers import PIPES, PIPE_SAMPLES, gpu_render, pkg, vertices_for
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _clip_scene(seed, n, spread, width, height):
    """Small clip-space triangles, a share of them crossing the frustum planes."""
    rng = np.random.default_rng(seed)
    w = rng.uniform(0.2, 10, size=(n * 3,)).astype(np.float32)
    c = rng.uniform(-spread, spread, size=(n, 3))
    off = rng.normal(0, 0.05, size=(n, 3, 3))
    ndc = (c[:, None, :] + off).reshape(-1, 3)
    v = np.zeros((n * 3, 8), np.float32)
    v[:, 0:3] = ndc * w[:, None]
    v[:, 3] = w
    v[:, 4:8] = rng.uniform(0, 1, size=(n * 3, 4))
    return {"vertices": v, "indices": np.arange(n * 3, dtype=np.int32).reshape(-1, 3), "width": width,
            "height": height}


def _near_clipped_soup():
    sc = pkg_mod("scenes").soup(4000, 256, 200, seed=9, median_px=400.0, sigma=1.2)
    v = sc["vertices"].copy()
    v[::7, 2] = -1.5 * v[::7, 3]   # through the near plane
    sc["vertices"] = v
    return sc


SCENES = {
    "soup": lambda: pkg_mod("scenes").soup(20000, 320, 240, seed=21, median_px=6.0),
    "near_clipped": _near_clipped_soup,
    "clip_planes": lambda: _clip_scene(22, 3000, 2.5, 640, 480),
}


@pytest.mark.parametrize("pipe", ["PixelPipe_gouraud", "PixelPipe_gouraud_msaa4", "PixelPipe_gouraud_flat"])
@pytest.mark.parametrize("scene", list(SCENES))
def test_setup_words_equal_oracle(cuda, pipe, scene):
    p = pkg()
    lib = pkg_mod("_lib").load()
    sc = SCENES[scene]()
    cr = p.CudaRaster()
    cr.init()
    clear = (p.color_to_abgr(0.1, 0.2, 0.3, 1.0), p.clear_depth_from_float(1.0))
    gpu_render(pipe, sc, clear, cr=cr)
    T = sc["indices"].shape[0]
    cap = T * 8 + 16
    sub = np.zeros(T, np.uint8)
    hdr = np.zeros((cap, 4), np.uint32)
    dat = np.zeros((cap, 16), np.uint32)
    nt, ns = C.c_int64(), C.c_int64()
    assert lib.cr_read_setup_output(cr._ctx, sub.ctypes.data, hdr.ctypes.data, dat.ctypes.data, cap, C.byref(nt),
                                    C.byref(ns)) == 0
    assert nt.value == T
    flags, _, _, stride = PIPES[pipe]
    op = orc.make_pipe(sc["width"], sc["height"], PIPE_SAMPLES.get(pipe, 1), flags, "replace", "gouraud", stride)
    osub, ohdr, odat, used = orc.setup(op, vertices_for(pipe, sc["vertices"]), sc["indices"], cap)
    assert used == ns.value
    assert np.array_equal(sub, osub)
    one = np.nonzero(osub == 1)[0]
    assert np.array_equal(hdr[one], ohdr[one]) and np.array_equal(dat[one], odat[one])
    multi = np.nonzero(osub > 1)[0]
    for t in multi:
        gb, ob, k = int(hdr[t, 3]), int(ohdr[t, 3]), int(osub[t])
        assert gb >= T and ob >= T
        assert np.array_equal(hdr[gb:gb + k], ohdr[ob:ob + k]), f"triangle {t}"
        assert np.array_equal(dat[gb:gb + k], odat[ob:ob + k]), f"triangle {t}"
    if scene != "soup":
        assert len(multi) > 0, "the scene should clip some triangles into several subtriangles"


def test_read_setup_output_validation(cuda):
    p = pkg()
    lib = pkg_mod("_lib").load()
    cr = p.CudaRaster()
    cr.init()
    nt, ns = C.c_int64(), C.c_int64()
    assert lib.cr_read_setup_output(cr._ctx, None, None, None, 0, C.byref(nt), C.byref(ns)) == 0
    assert nt.value == 0 and ns.value == 0
    sc = pkg_mod("scenes").soup(100, 64, 64, seed=3)
    clear = (p.color_to_abgr(0.0, 0.0, 0.0, 1.0), p.clear_depth_from_float(1.0))
    gpu_render("PixelPipe_gouraud", sc, clear, cr=cr)
    buf = np.zeros((8, 4), np.uint32)
    assert lib.cr_read_setup_output(cr._ctx, None, buf.ctypes.data, None, 8, C.byref(nt), C.byref(ns)) == 5
    assert lib.cr_read_setup_output(cr._ctx, None, None, None, -1, C.byref(nt), C.byref(ns)) == 1
