"""cr_draw_triangles_static: the draw for callers that may not allocate memory
while they run (a host that owns a fixed memory budget, a real-time loop
where cudaMalloc would stall the frame, a plugin that only gets device
pointers). Its queues live in a static device array inside the library.

The test calls it through the C ABI twice in a row on fresh surfaces and
checks both framebuffers against the ordinary context-based draw
(cr_draw_triangles), bit for bit like every other parity test, plus the
limits it must reject. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import pkg_mod
from helpers import PIPE_SAMPLES, assert_same, gpu_render, vertices_for

pytestmark = pytest.mark.gpu

CR_OK, CR_ERR_CAPACITY = 0, 5


def _static_fn():
    lib = pkg_mod("_lib").load()
    fn = lib.cr_draw_triangles_static
    fn.restype = C.c_int
    fn.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                   C.c_int32, C.c_int32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_char_p, C.c_int64]
    return fn


def _draw_static(fn, pipe, sc, clear, torch):
    samples = PIPE_SAMPLES.get(pipe, 1)
    w, h = sc["width"], sc["height"]
    rows, words = (h + 7) & ~7, ((w + 7) & ~7) * samples
    color = torch.zeros((rows, words), dtype=torch.int32, device="cuda")
    depth = torch.zeros((rows, words), dtype=torch.int32, device="cuda")
    verts = torch.from_numpy(vertices_for(pipe, sc["vertices"])).cuda()
    idx = torch.from_numpy(np.ascontiguousarray(sc["indices"], dtype=np.int32)).cuda()
    err = C.create_string_buffer(512)
    stream = torch.cuda.current_stream().cuda_stream
    st = fn(pipe.encode(), color.data_ptr(), depth.data_ptr(), w, h, samples, verts.data_ptr(), idx.data_ptr(),
            idx.shape[0], 1, clear[0], clear[1], C.c_void_p(stream), err, len(err))
    assert st == CR_OK, err.value.decode()
    torch.cuda.synchronize()
    to_u32 = lambda t: (t.cpu().numpy().view(np.uint32)).copy()
    return to_u32(color), to_u32(depth)


@pytest.mark.parametrize("pipe,scene", [("PixelPipe_gouraud", "soup"), ("PixelPipe_gouraud_srcover", "soup"),
                                        ("PixelPipe_gouraud_msaa4", "soup"), ("PixelPipe_gouraud", "cube")])
def test_static_draw_matches_context_draw(cuda, pipe, scene):
    scenes = pkg_mod("scenes")
    sc = scenes.cube(640, 480) if scene == "cube" else scenes.soup(20000, 320, 240, seed=4, median_px=6.0)
    p = pkg_mod("raster")
    clear = (p.color_to_abgr(0.2, 0.4, 0.8, 1.0), p.clear_depth_from_float(1.0))
    ref_c, ref_d, _, _ = gpu_render(pipe, sc, clear)
    fn = _static_fn()
    for call in range(2):
        c, d = _draw_static(fn, pipe, sc, clear, cuda)
        assert_same(c, d, ref_c, ref_d, f"{pipe} static call {call + 1}")


def test_static_draw_rejects_oversize(cuda):
    fn = _static_fn()
    err = C.create_string_buffer(512)
    dummy = cuda.zeros(16, dtype=cuda.int32, device="cuda")
    ptr = dummy.data_ptr()
    st = fn(b"PixelPipe_gouraud", ptr, ptr, 64, 64, 1, ptr, ptr, 65537, 1, 0, 0, None, err, len(err))
    assert st == CR_ERR_CAPACITY and b"65536" in err.value
    st = fn(b"PixelPipe_gouraud", ptr, ptr, 2000, 64, 1, ptr, ptr, 1, 1, 0, 0, None, err, len(err))
    assert st == CR_ERR_CAPACITY and b"1024" in err.value
