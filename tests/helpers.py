"""Shared helpers for the GPU parity tests: render a scene through the C ABI
(via the Python mirror of the reference API) and through the CPU oracle."""
from __future__ import annotations

import importlib

import numpy as np

from oracle import oracle as orc

PKG = "cudaraster-linux_gb300"

# pipe name -> (oracle flags, blend, shader, vertex stride)
PIPES = {
    "PixelPipe_gouraud": (orc.DEPTH | orc.LERP, "replace", "gouraud", 32),
    "PixelPipe_gouraud_srcover": (orc.DEPTH | orc.LERP, "srcover", "gouraud", 32),
    "PixelPipe_passthrough": (orc.DEPTH | orc.LERP, "replace", "red", 16),
    "PixelPipe_gouraud_additive": (orc.DEPTH | orc.LERP, "additive", "gouraud", 32),
    "PixelPipe_gouraud_depthonly": (orc.DEPTH | orc.LERP, "depthonly", "gouraud", 32),
    "PixelPipe_gouraud_nodepth": (orc.LERP, "srcover", "gouraud", 32),
    "PixelPipe_gouraud_flat": (orc.DEPTH, "replace", "gouraud", 32),
    "PixelPipe_trihash_srcover": (0, "srcover", "trihash", 32),
    "PixelPipe_deriv_quads": (orc.DEPTH | orc.LERP | orc.QUADS, "replace", "deriv", 32),
    "PixelPipe_gouraud_msaa2": (orc.DEPTH | orc.LERP, "replace", "gouraud", 32),
    "PixelPipe_gouraud_msaa4": (orc.DEPTH | orc.LERP, "replace", "gouraud", 32),
    "PixelPipe_gouraud_msaa8": (orc.DEPTH | orc.LERP, "replace", "gouraud", 32),
    "PixelPipe_gouraud_srcover_msaa4": (orc.DEPTH | orc.LERP, "srcover", "gouraud", 32),
    "PixelPipe_trihash_srcover_msaa4": (0, "srcover", "trihash", 32),
    "PixelPipe_texPhong": (orc.DEPTH | orc.LERP, "replace", "texphong", 64),
    "PixelPipe_texPhong_quads": (orc.DEPTH | orc.LERP | orc.QUADS, "replace", "texphong", 64),
    "PixelPipe_texPhong_srcover": (orc.DEPTH | orc.LERP, "srcover", "texphong", 64),
    "PixelPipe_texPhong_msaa4": (orc.DEPTH | orc.LERP, "replace", "texphong", 64),
}
PIPE_SAMPLES = {"PixelPipe_gouraud_msaa2": 2, "PixelPipe_gouraud_msaa4": 4, "PixelPipe_gouraud_msaa8": 8,
                "PixelPipe_gouraud_srcover_msaa4": 4, "PixelPipe_trihash_srcover_msaa4": 4,
                "PixelPipe_texPhong_msaa4": 4}


def pkg():
    return importlib.import_module(PKG)


def vertices_for(pipe: str, verts: np.ndarray) -> np.ndarray:
    stride = PIPES[pipe][3]
    # The pipe reads stride bytes per vertex: a narrower array would be read past its end.
    assert verts.ndim == 2 and verts.shape[1] * 4 >= stride, f"{pipe} needs {stride}-byte vertex records"
    return np.ascontiguousarray(verts[:, : stride // 4], dtype=np.float32)


def oracle_render(pipe: str, sc: dict, clear=None, color=None, depth=None, threads: int = 0):
    flags, blend, shader, stride = PIPES[pipe]
    samples = PIPE_SAMPLES.get(pipe, 1)
    p = orc.make_pipe(sc["width"], sc["height"], samples, flags, blend, shader, stride, clear)
    return orc.render(p, vertices_for(pipe, sc["vertices"]), sc["indices"], color, depth, threads)


def init_surfaces(sc: dict, samples: int, seed: int | None):
    shape = orc.surface_shape(sc["width"], sc["height"], samples)
    if seed is None:
        return np.zeros(shape, np.uint32), np.zeros(shape, np.uint32)
    rng = np.random.default_rng(seed)
    return (rng.integers(0, 2**32, shape, dtype=np.uint64).astype(np.uint32),
            rng.integers(0, 2**32, shape, dtype=np.uint64).astype(np.uint32))


def gpu_render(pipe: str, sc: dict, clear=None, color=None, depth=None, cr=None, tuning=None, capacity=None,
               num_tris=None):
    """Returns (color, depth, counters, stats). clear=(abgr, encoded depth) or None."""
    import torch
    p = pkg()
    samples = PIPE_SAMPLES.get(pipe, 1)
    w, h = sc["width"], sc["height"]
    if cr is None:
        cr = p.CudaRaster()
        cr.init()
    if tuning:
        cr.setTuning(**tuning)
    if capacity:
        cr.setCapacity(*capacity)
    cs = p.CudaSurface((w, h), p.CudaSurface.FORMAT_RGBA8, samples)
    ds = p.CudaSurface((w, h), p.CudaSurface.FORMAT_DEPTH32, samples)
    if color is not None:
        cs.tensor.copy_(torch.from_numpy(color.view(np.int32)))
        ds.tensor.copy_(torch.from_numpy(depth.view(np.int32)))
    cr.setSurfaces(cs, ds)
    cr.setPixelPipe(None, pipe)
    verts = torch.from_numpy(vertices_for(pipe, sc["vertices"])).cuda()
    idx = torch.from_numpy(np.ascontiguousarray(sc["indices"], dtype=np.int32)).cuda()
    if clear is not None:
        cr._check(cr._lib.cr_deferred_clear_raw(cr._ctx, clear[0], clear[1]))
    cr.setVertexBuffer(verts, 0)
    cr.setIndexBuffer(idx, 0, idx.shape[0] if num_tris is None else num_tris)
    cr.drawTriangles()
    torch.cuda.synchronize()
    gc = cs.download().numpy().astype(np.uint32)
    gd = ds.download().numpy().astype(np.uint32)
    return gc, gd, cr.getCounters(), cr.getStats()


def assert_same(gpu_c, gpu_d, ref_c, ref_d, what=""):
    bc = np.argwhere(gpu_c != ref_c)
    bd = np.argwhere(gpu_d != ref_d)
    msg = f"{what}: colour mismatches {len(bc)}, depth mismatches {len(bd)}"
    if len(bc):
        y, x = bc[0]
        msg += f"; first colour at row {y} word {x}: gpu {gpu_c[y, x]:#010x} oracle {ref_c[y, x]:#010x}"
    if len(bd):
        y, x = bd[0]
        msg += f"; first depth at row {y} word {x}: gpu {gpu_d[y, x]:#010x} oracle {ref_d[y, x]:#010x}"
    assert len(bc) == 0 and len(bd) == 0, msg
