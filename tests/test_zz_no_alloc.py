"""cr_draw_triangles_static: the draw for callers that may not allocate memory
while they run (a host that owns a fixed memory budget, a real-time loop
where cudaMalloc would stall the frame, a plugin that only gets device
pointers). Its queues live in a static device array inside the library.

The test calls it through the C ABI twice in a row on fresh surfaces and
checks both framebuffers against the ordinary context-based draw
(cr_draw_triangles) and against the CPU oracle, bit for bit like every other
parity test; then the limits it must reject, a draw inside the limits that
overflows the fixed queues (CR_ERR_CAPACITY, surfaces untouched, the next call
exact again) and a draw of no triangles with a deferred clear. This file is
collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import pkg_mod
from helpers import PIPE_SAMPLES, assert_same, gpu_render, init_surfaces, oracle_render, vertices_for

pytestmark = pytest.mark.gpu

CR_OK, CR_ERR_CAPACITY = 0, 5


def _static_fn():
    lib = pkg_mod("_lib").load()
    fn = lib.cr_draw_triangles_static
    fn.restype = C.c_int
    fn.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                   C.c_int32, C.c_int32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_char_p, C.c_int64]
    return fn


def _draw_static(fn, pipe, sc, clear, torch, init=None, expect=CR_OK, num_tris=None):
    """One static draw on fresh surfaces (or on copies of init = (colour, depth));
    returns the surfaces and the error text."""
    samples = PIPE_SAMPLES.get(pipe, 1)
    w, h = sc["width"], sc["height"]
    rows, words = (h + 7) & ~7, ((w + 7) & ~7) * samples
    if init is None:
        color = torch.zeros((rows, words), dtype=torch.int32, device="cuda")
        depth = torch.zeros((rows, words), dtype=torch.int32, device="cuda")
    else:
        color = torch.from_numpy(init[0].view(np.int32).copy()).cuda()
        depth = torch.from_numpy(init[1].view(np.int32).copy()).cuda()
    verts = torch.from_numpy(vertices_for(pipe, sc["vertices"])).cuda()
    idx = torch.from_numpy(np.ascontiguousarray(sc["indices"], dtype=np.int32)).cuda()
    err = C.create_string_buffer(512)
    stream = torch.cuda.current_stream().cuda_stream
    n = idx.shape[0] if num_tris is None else num_tris
    st = fn(pipe.encode(), color.data_ptr(), depth.data_ptr(), w, h, samples, verts.data_ptr(), idx.data_ptr(),
            n, 1 if clear is not None else 0, clear[0] if clear else 0, clear[1] if clear else 0,
            C.c_void_p(stream), err, len(err))
    assert st == expect, f"status {st}: {err.value.decode()}"
    torch.cuda.synchronize()
    to_u32 = lambda t: (t.cpu().numpy().view(np.uint32)).copy()
    return to_u32(color), to_u32(depth), err.value.decode()


@pytest.mark.parametrize("pipe,scene", [("PixelPipe_gouraud", "soup"), ("PixelPipe_gouraud_srcover", "soup"),
                                        ("PixelPipe_gouraud_msaa4", "soup"), ("PixelPipe_gouraud", "cube")])
def test_static_draw_matches_context_draw(cuda, pipe, scene):
    scenes = pkg_mod("scenes")
    sc = scenes.cube(640, 480) if scene == "cube" else scenes.soup(20000, 320, 240, seed=4, median_px=6.0)
    p = pkg_mod("raster")
    clear = (p.color_to_abgr(0.2, 0.4, 0.8, 1.0), p.clear_depth_from_float(1.0))
    ref_c, ref_d, _, _ = gpu_render(pipe, sc, clear)
    orc_c, orc_d, st = oracle_render(pipe, sc, clear)
    assert st["zmin_violations"] == 0
    fn = _static_fn()
    for call in range(2):
        c, d, _ = _draw_static(fn, pipe, sc, clear, cuda)
        assert_same(c, d, ref_c, ref_d, f"{pipe} static call {call + 1} vs cr_draw_triangles")
        assert_same(c, d, orc_c, orc_d, f"{pipe} static call {call + 1} vs oracle")


def _full_screen_quads(n_quads, width, height, seed):
    """n_quads screen-filling quads (two triangles each, inside the clip volume so
    none is clipped) at random depths, with random colours: every quad puts an
    entry in every 8x8 tile of the viewport."""
    rng = np.random.default_rng(seed)
    verts, idx = [], []
    for q in range(n_quads):
        z = rng.uniform(-0.9, 0.9)
        w = rng.uniform(1.0, 3.0)
        base = len(verts)
        for x, y in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
            verts.append([x * w, y * w, z * w, w, *rng.uniform(0.0, 1.0, 4)])
        idx += [[base, base + 1, base + 2], [base, base + 2, base + 3]]
    return {"vertices": np.array(verts, np.float32), "indices": np.array(idx, np.int32), "width": width,
            "height": height}


def test_static_draw_queue_overflow_leaves_surfaces_and_recovers(cuda):
    """Inside the argument limits but beyond the fixed tile queue (16 entries per
    allowed triangle, 1,048,576): 100 full-screen quads at 1024x1024 need about
    1.7M tile entries. The call must fail with CR_ERR_CAPACITY and leave the
    pre-filled surfaces as they were; a following call that fits must be exact."""
    fn = _static_fn()
    pipe = "PixelPipe_gouraud"
    big = _full_screen_quads(100, 1024, 1024, seed=21)
    c0, d0 = init_surfaces(big, 1, seed=22)
    p = pkg_mod("raster")
    clear = (p.color_to_abgr(0.2, 0.4, 0.8, 1.0), p.clear_depth_from_float(1.0))
    c, d, err = _draw_static(fn, pipe, big, clear, cuda, init=(c0, d0), expect=CR_ERR_CAPACITY)
    assert "static queues" in err
    assert np.array_equal(c, c0) and np.array_equal(d, d0), "an overflowing static draw changed the surfaces"
    small = pkg_mod("scenes").soup(20000, 1024, 1024, seed=23, median_px=6.0)
    orc_c, orc_d, _ = oracle_render(pipe, small, clear)
    for call in range(2):
        c, d, _ = _draw_static(fn, pipe, small, clear, cuda)
        assert_same(c, d, orc_c, orc_d, f"static call {call + 1} after an overflow")


def test_static_draw_no_triangles_clears(cuda):
    """num_tris = 0 with a deferred clear: every sample takes the clear values."""
    fn = _static_fn()
    sc = pkg_mod("scenes").soup(100, 200, 120, seed=24)
    p = pkg_mod("raster")
    clear = (p.color_to_abgr(0.3, 0.5, 0.7, 1.0), p.clear_depth_from_float(0.75))
    c0, d0 = init_surfaces(sc, 4, seed=25)
    c, d, _ = _draw_static(fn, "PixelPipe_gouraud_msaa4", sc, clear, cuda, init=(c0, d0), num_tris=0)
    orc_c, orc_d, _ = oracle_render("PixelPipe_gouraud_msaa4", dict(sc, indices=sc["indices"][:0]), clear,
                                    c0.copy(), d0.copy())
    assert_same(c, d, orc_c, orc_d, "static draw of no triangles")
    assert (c[:120, : 200 * 4] == clear[0]).all() and (d[:120, : 200 * 4] == clear[1]).all()


def test_static_draw_rejects_oversize(cuda):
    fn = _static_fn()
    err = C.create_string_buffer(512)
    dummy = cuda.zeros(16, dtype=cuda.int32, device="cuda")
    ptr = dummy.data_ptr()
    st = fn(b"PixelPipe_gouraud", ptr, ptr, 64, 64, 1, ptr, ptr, 65537, 1, 0, 0, None, err, len(err))
    assert st == CR_ERR_CAPACITY and b"65536" in err.value
    st = fn(b"PixelPipe_gouraud", ptr, ptr, 2000, 64, 1, ptr, ptr, 1, 1, 0, 0, None, err, len(err))
    assert st == CR_ERR_CAPACITY and b"1024" in err.value
