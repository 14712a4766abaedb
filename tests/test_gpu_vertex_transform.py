"""The vertex transform fused into setup (cr_set_vertex_transform): the same
framebuffers, bit for bit, as running vertexShader_passthrough first and
drawing its records, and as the CPU oracle -- triangles crossing the near
plane (the clip path) included."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import pkg_mod
from helpers import assert_same, oracle_render, pkg
from oracle import vertex_oracle as vo

pytestmark = pytest.mark.gpu


def _draw(pipe, samples, model, colors, idx, mvp, w, h, fused, model_stride4=False):
    p = pkg()
    raster = pkg_mod("raster")
    cr = p.CudaRaster()
    cr.init()
    cs = p.CudaSurface((w, h), p.CudaSurface.FORMAT_RGBA8, samples)
    ds = p.CudaSurface((w, h), p.CudaSurface.FORMAT_DEPTH32, samples)
    cr.setSurfaces(cs, ds)
    cr.setPixelPipe(None, pipe)
    m = torch.from_numpy(model).cuda()
    c = torch.from_numpy(colors).cuda()
    if fused:
        rec = torch.zeros((model.shape[0], 8), dtype=torch.float32, device="cuda")
        rec[:, 4:8] = c
        if model_stride4:
            m4 = torch.ones((model.shape[0], 4), dtype=torch.float32, device="cuda")
            m4[:, 0:3] = m
            m = m4
        cr.setVertexTransform(m, mvp)
    else:
        rec = raster.vertex_shader_passthrough(m, mvp, c)
    cr.setVertexBuffer(rec, 0)
    ib = torch.from_numpy(np.ascontiguousarray(idx, dtype=np.int32)).cuda()
    cr.setIndexBuffer(ib, 0, ib.shape[0])
    cr.deferredClear((0.1, 0.3, 0.5, 1.0), 1.0)
    cr.drawTriangles()
    torch.cuda.synchronize()
    return cs.download().numpy().astype(np.uint32), ds.download().numpy().astype(np.uint32), (cr, cs, ds)


def _terrain(n, seed, frame, w, h, elevation=15.0):
    scenes = pkg_mod("scenes")
    pos, rgba, tris = scenes.grid_mesh(n, seed)
    eye, target = scenes.terrain_eye_target(frame, elevation)
    # A near plane at 0.3 cuts through the heightfield in front of the camera: the clip path runs.
    mvp = (scenes.perspective(60.0, w / h, 0.3, 10.0) @ scenes.look_at(eye * 0.35, target)).astype(np.float32)
    return pos.astype(np.float32), rgba.astype(np.float32), tris, mvp


@pytest.mark.parametrize("pipe,samples", [("PixelPipe_gouraud", 1), ("PixelPipe_gouraud_msaa4", 4),
                                          ("PixelPipe_gouraud_srcover", 1)])
def test_fused_equals_vertex_stage_and_oracle(cuda, pipe, samples):
    p = pkg()
    w, h = 800, 600
    pos, rgba, tris, mvp = _terrain(256, 4, 30.0, w, h)
    fc, fd, _ = _draw(pipe, samples, pos, rgba, tris, mvp, w, h, fused=True)
    uc, ud, _ = _draw(pipe, samples, pos, rgba, tris, mvp, w, h, fused=False)
    assert_same(fc, fd, uc, ud, "fused vs vertex stage")
    verts = np.concatenate([vo.vertex_passthrough(pos, mvp), rgba], axis=1).astype(np.float32)
    clear = (p.color_to_abgr(0.1, 0.3, 0.5, 1.0), p.clear_depth_from_float(1.0))
    rc, rd, st = oracle_render(pipe, {"vertices": verts, "indices": tris, "width": w, "height": h}, clear)
    assert st["zmin_violations"] == 0
    assert st["num_clipped"] > 0, "camera inside the geometry should clip some triangles"
    assert_same(fc, fd, rc, rd, "fused vs oracle")


def test_fused_padded_model_and_turning_off(cuda):
    raster = pkg_mod("raster")
    w, h = 640, 480
    pos, rgba, tris, mvp = _terrain(128, 6, 80.0, w, h)
    a = _draw("PixelPipe_gouraud", 1, pos, rgba, tris, mvp, w, h, fused=True, model_stride4=True)
    b = _draw("PixelPipe_gouraud", 1, pos, rgba, tris, mvp, w, h, fused=False)
    assert_same(a[0], a[1], b[0], b[1], "stride-4 model")
    # Turned off, setup reads the records' clip positions again.
    cr, cs, ds = a[2]
    cr.setVertexTransform(None)
    rec = raster.vertex_shader_passthrough(torch.from_numpy(pos).cuda(), mvp, torch.from_numpy(rgba).cuda())
    cr.setVertexBuffer(rec, 0)
    cr.deferredClear((0.1, 0.3, 0.5, 1.0), 1.0)
    cr.drawTriangles()
    torch.cuda.synchronize()
    c = cs.download().numpy().astype(np.uint32)
    d = ds.download().numpy().astype(np.uint32)
    assert_same(c, d, b[0], b[1], "transform off")


def test_vertex_transform_validation(cuda):
    p = pkg()
    lib = pkg_mod("_lib").load()
    cr = p.CudaRaster()
    cr.init()
    m = torch.zeros((4, 3), dtype=torch.float32, device="cuda")
    mvp = (ctypes.c_float * 16)(*([1.0] + [0.0] * 15))
    assert lib.cr_set_vertex_transform(cr._ctx, m.data_ptr(), 3, mvp) == 0
    assert lib.cr_set_vertex_transform(cr._ctx, m.data_ptr(), 2, mvp) == 1
    assert lib.cr_set_vertex_transform(cr._ctx, m.data_ptr(), 3, None) == 1
    assert lib.cr_set_vertex_transform(cr._ctx, m.data_ptr() + 2, 3, mvp) == 1
    assert lib.cr_set_vertex_transform(cr._ctx, None, 0, None) == 0
