"""GPU framebuffers against the CPU oracle, bit for bit (colour and depth, every
pixel and sample), through the C ABI."""
import numpy as np
import pytest

from helpers import PIPES, PIPE_SAMPLES, assert_same, gpu_render, init_surfaces, oracle_render, pkg
from conftest import pkg_mod

pytestmark = pytest.mark.gpu


def clear_of(rgba=(0.2, 0.4, 0.8, 1.0), depth=1.0):
    p = pkg()
    return (p.color_to_abgr(*rgba), p.clear_depth_from_float(depth))


def test_cube_config1(cuda):
    sc = pkg_mod("scenes").cube(1024, 768)
    clear = clear_of()
    gc, gd, cnt, _ = gpu_render("PixelPipe_gouraud", sc, clear)
    rc, rd, st = oracle_render("PixelPipe_gouraud", sc, clear)
    assert st["zmin_violations"] == 0
    assert_same(gc, gd, rc, rd, "cube")
    assert (rc != clear[0]).sum() > 100000


# Pipes that draw the soup's GouraudVertex records (the textured pipes have their own tests).
@pytest.mark.parametrize("pipe", [p for p in PIPES if p not in PIPE_SAMPLES and p != "PixelPipe_deriv_quads"
                                  and PIPES[p][3] <= 32])
def test_soup_pipes(cuda, pipe):
    sc = pkg_mod("scenes").soup(20000, 320, 240, seed=11, median_px=6.0)
    clear = clear_of()
    gc, gd, _, _ = gpu_render(pipe, sc, clear)
    rc, rd, st = oracle_render(pipe, sc, clear)
    assert st["zmin_violations"] == 0
    assert_same(gc, gd, rc, rd, pipe)


@pytest.mark.parametrize("median_px,seed", [(3.0, 12), (9.0, 13), (40.0, 14)])
def test_quad_derivatives(cuda, median_px, seed):
    # Quad mode: derivatives across each 2x2 quad, helper pixels shaded but not written.
    sc = pkg_mod("scenes").soup(6000, 256, 184, seed=seed, median_px=median_px)
    clear = clear_of()
    gc, gd, _, _ = gpu_render("PixelPipe_deriv_quads", sc, clear)
    rc, rd, st = oracle_render("PixelPipe_deriv_quads", sc, clear)
    assert st["zmin_violations"] == 0
    assert_same(gc, gd, rc, rd, "deriv quads")
    assert len(np.unique(rc)) > 100   # the derivatives vary across the frame


def test_quad_derivatives_cube(cuda):
    sc = pkg_mod("scenes").cube(640, 480)
    clear = clear_of()
    gc, gd, _, _ = gpu_render("PixelPipe_deriv_quads", sc, clear)
    rc, rd, _ = oracle_render("PixelPipe_deriv_quads", sc, clear)
    assert_same(gc, gd, rc, rd, "deriv quads cube")


@pytest.mark.parametrize("pipe", [p for p in PIPE_SAMPLES if PIPES[p][3] <= 32])
def test_soup_msaa(cuda, pipe):
    sc = pkg_mod("scenes").soup(8000, 200, 136, seed=5, median_px=5.0)
    sc["samples"] = PIPE_SAMPLES[pipe]
    clear = clear_of((0.1, 0.1, 0.1, 1.0), 1.0)
    gc, gd, _, _ = gpu_render(pipe, sc, clear)
    rc, rd, st = oracle_render(pipe, sc, clear)
    assert st["zmin_violations"] == 0
    assert_same(gc, gd, rc, rd, pipe)


def test_no_clear_preserves_untouched(cuda):
    sc = pkg_mod("scenes").soup(3000, 197, 131, seed=3)
    c0, d0 = init_surfaces(sc, 1, seed=7)
    gc, gd, _, _ = gpu_render("PixelPipe_gouraud_srcover", sc, None, c0.copy(), d0.copy())
    rc, rd, _ = oracle_render("PixelPipe_gouraud_srcover", sc, None, c0.copy(), d0.copy())
    assert_same(gc, gd, rc, rd, "no clear")


def test_clipping_heavy(cuda):
    sc = pkg_mod("scenes").soup(4000, 256, 200, seed=9, median_px=400.0, sigma=1.2)
    # push a fraction of the triangles through the near plane
    v = sc["vertices"].copy()
    v[::7, 2] = -1.5 * v[::7, 3]
    sc["vertices"] = v
    clear = clear_of()
    gc, gd, cnt, _ = gpu_render("PixelPipe_gouraud", sc, clear)
    rc, rd, st = oracle_render("PixelPipe_gouraud", sc, clear)
    assert st["num_clipped"] > 0
    assert_same(gc, gd, rc, rd, "clipping")


def test_empty_draw_clears(cuda):
    """A draw without triangles still applies the deferred clear to every tile."""
    sc = pkg_mod("scenes").soup(10, 64, 40, seed=1)
    c0, d0 = init_surfaces(sc, 1, seed=3)
    clear = clear_of((0.5, 0.25, 0.125, 1.0), 0.5)
    gc, gd, _, _ = gpu_render("PixelPipe_gouraud", sc, clear, c0.copy(), d0.copy(), num_tris=0)
    empty = dict(sc, indices=sc["indices"][:0])
    rc, rd, _ = oracle_render("PixelPipe_gouraud", empty, clear, c0.copy(), d0.copy())
    assert_same(gc, gd, rc, rd, "empty draw")
    assert (gc == clear[0]).all() and (gd == clear[1]).all()
