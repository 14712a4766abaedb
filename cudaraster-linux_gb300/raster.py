"""Python mirror of the reference's host API (src/cudaraster/CudaRaster.hpp,
CudaSurface.hpp, framework/gpu/Buffer.hpp), over the C ABI.

Same class and method names, argument meaning and error behaviour (errors
raise RasterError where the reference calls fail()). PyTorch only provides
device memory and streams.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import _lib
from ._lib import RENDER_DEPTH, RENDER_LERP, RENDER_QUADS, RasterError, check  # noqa: F401


class Buffer:
    """Device buffer (the reference's Buffer, Buffer.hpp:39-158), backed by a torch tensor."""

    def __init__(self, tensor: torch.Tensor | None = None):
        self.tensor = tensor

    @classmethod
    def from_host(cls, array, device: str | torch.device = "cuda") -> "Buffer":
        t = torch.as_tensor(array)
        return cls(t.to(device).contiguous())

    def resizeDiscard(self, num_bytes: int, device: str | torch.device = "cuda") -> None:
        if self.tensor is None or self.tensor.numel() * self.tensor.element_size() < num_bytes:
            self.tensor = torch.empty(num_bytes, dtype=torch.uint8, device=device)

    def getCudaPtr(self, ofs: int = 0) -> int:
        return self.tensor.data_ptr() + ofs

    def getSize(self) -> int:
        return self.tensor.numel() * self.tensor.element_size()


class CudaSurface:
    """RGBA8 or DEPTH32 render target (CudaSurface.hpp:36-78) as a headless
    device buffer in the reference layout: rounded_h rows of rounded_w *
    numSamples words, sample i of pixel (x, y) at word
    y * rowWords + (x // 8) * 8 * numSamples + i * 8 + x % 8."""

    FORMAT_RGBA8 = 0
    FORMAT_DEPTH32 = 1

    def __init__(self, size, fmt: int, numSamples: int = 1, device: str | torch.device = "cuda"):
        w, h = int(size[0]), int(size[1])
        if min(w, h) <= 0:
            raise RasterError(1, "CudaSurface: Size must be positive!")
        if max(w, h) > 4095:
            raise RasterError(5, "CudaSurface: CR_MAXVIEWPORT_SIZE exceeded!")
        if fmt not in (self.FORMAT_RGBA8, self.FORMAT_DEPTH32):
            raise RasterError(1, "CudaSurface: Invalid format!")
        if numSamples > 8:
            raise RasterError(1, "CudaSurface: numSamples cannot exceed 8!")
        if numSamples < 1 or (numSamples & (numSamples - 1)):
            raise RasterError(1, "CudaSurface: numSamples must be a power of two!")
        self.size = (w, h)
        self.roundedSize = ((w + 7) & ~7, (h + 7) & ~7)
        self.textureSize = (self.roundedSize[0] * numSamples, self.roundedSize[1])
        self.format = fmt
        self.numSamples = numSamples
        self.tensor = torch.zeros((self.textureSize[1], self.textureSize[0]), dtype=torch.int32, device=device)

    def getSize(self):
        return self.size

    def getRoundedSize(self):
        return self.roundedSize

    def getTextureSize(self):
        return self.textureSize

    def getFormat(self):
        return self.format

    def getNumSamples(self):
        return self.numSamples

    def getSamplesLog2(self):
        return self.numSamples.bit_length() - 1

    def getDevicePtr(self) -> int:
        return self.tensor.data_ptr()

    def download(self) -> torch.Tensor:
        """Raw words (uint32 values in an int64 tensor), shape (rows, rowWords)."""
        return self.tensor.cpu().to(torch.int64) & 0xFFFFFFFF

    def resolve(self, stream: torch.cuda.Stream | None = None) -> torch.Tensor:
        """MSAA resolve of a colour surface (cr_resolve_color): a (height,
        width, 4) uint8 tensor on the device, channels R, G, B, A."""
        if self.getFormat() != self.FORMAT_RGBA8:
            raise RasterError(1, "CudaSurface: only colour surfaces resolve")
        w, h = self.getSize()
        out = torch.empty((h, w, 4), dtype=torch.uint8, device=self.tensor.device)
        s = (stream or torch.cuda.current_stream()).cuda_stream
        check(_lib.load().cr_resolve_color(self.getDevicePtr(), w, h, self.getNumSamples(), out.data_ptr(), w * 4,
                                           C.c_void_p(s)))
        return out

    def fill(self, value: int) -> None:
        v = value - (1 << 32) if value >= (1 << 31) else value
        self.tensor.fill_(v)


@dataclass
class Stats:
    setupTime: float
    binTime: float
    coarseTime: float
    fineTime: float


@dataclass
class DebugParams:
    emulateTriangleSetup: bool = False
    emulateBinRaster: bool = False
    emulateCoarseRaster: bool = False
    emulateFineRaster: bool = False


def pipe_names() -> list[str]:
    lib = _lib.load()
    out = []
    for i in range(lib.cr_pipe_count()):
        info = _lib.PipeInfo()
        check(lib.cr_pipe_info_at(i, C.byref(info)))
        out.append(info.name.decode())
    return out


def pipe_info(name: str) -> _lib.PipeInfo:
    lib = _lib.load()
    info = _lib.PipeInfo()
    check(lib.cr_pipe_info_by_name(name.encode(), C.byref(info)))
    return info


class CudaRaster:
    """The reference's CudaRaster (CudaRaster.hpp:42-190)."""

    Stats = Stats
    DebugParams = DebugParams

    def __init__(self):
        self._lib = _lib.load()
        self._ctx = None
        self._keep = []

    # CudaRaster.cpp:98-128
    def init(self) -> None:
        ctx = C.c_void_p()
        st = self._lib.cr_create(C.byref(ctx))
        if st != _lib.CR_OK:
            raise RasterError(st, "CudaRaster: No CUDA-capable devices found!" if st == 6 else
                              "CudaRaster: Compute capability 10.x or better is required!")
        self._ctx = ctx

    def __del__(self):
        if getattr(self, "_ctx", None):
            try:
                self._lib.cr_destroy(self._ctx)
            except Exception:
                pass
            self._ctx = None

    def _check(self, st: int) -> None:
        check(st, self._ctx)

    def _need_init(self):
        if not self._ctx:
            raise RasterError(2, "CudaRaster: not initialized!")

    def setSurfaces(self, color: CudaSurface | None, depth: CudaSurface | None) -> None:
        self._need_init()
        if color is None and depth is None:
            self._check(self._lib.cr_set_surfaces(self._ctx, None, None, 0, 0, 0))
            return
        if color is None:
            raise RasterError(1, "CudaRaster: No color buffer specified!")
        if depth is None:
            raise RasterError(1, "CudaRaster: No depth buffer specified!")
        if color.getFormat() != CudaSurface.FORMAT_RGBA8:
            raise RasterError(1, "CudaRaster: Unsupported color buffer format!")
        if depth.getFormat() != CudaSurface.FORMAT_DEPTH32:
            raise RasterError(1, "CudaRaster: Unsupported depth buffer format!")
        if color.getSize() != depth.getSize():
            raise RasterError(1, "CudaRaster: Mismatch in size between surfaces!")
        if color.getNumSamples() != depth.getNumSamples():
            raise RasterError(1, "CudaRaster: Mismatch in multisampling between surfaces!")
        self._surfaces = (color, depth)
        w, h = color.getSize()
        self._check(self._lib.cr_set_surfaces(self._ctx, color.getDevicePtr(), depth.getDevicePtr(), w, h,
                                              color.getNumSamples()))

    def deferredClear(self, color=(0.0, 0.0, 0.0, 0.0), depth: float = 1.0) -> None:
        self._need_init()
        if not hasattr(color, "__len__"):
            color = (float(color),) * 4
        r, g, b, a = (float(c) for c in color)
        self._check(self._lib.cr_deferred_clear(self._ctx, r, g, b, a, float(depth)))

    def setPixelPipe(self, module, name: str | None = None) -> None:
        """setPixelPipe(module, name) as the reference; `module` is accepted for
        signature compatibility (pipes are compiled into the library) and may be None.
        setPixelPipe(name) is also accepted."""
        self._need_init()
        if name is None and isinstance(module, str):
            name = module
        self._check(self._lib.cr_set_pixel_pipe(self._ctx, name.encode() if name else None))

    def setVertexBuffer(self, buf, ofs: int = 0) -> None:
        self._need_init()
        ptr = _ptr_of(buf)
        self._vb = buf
        self._check(self._lib.cr_set_vertex_buffer(self._ctx, ptr, int(ofs)))

    def setVertexTransform(self, model: torch.Tensor | None, mvp=None) -> None:
        """Fuses vertexShader_passthrough into setup: while set, drawTriangles takes each
        vertex's clip position as mvp * (model[i, :3], 1) (same bits as running the shader
        first) and reads only the varyings from the vertex buffer. model: [N, >=3] float32
        CUDA tensor (kept alive here); mvp: 16 values, row-major. None turns it off."""
        self._need_init()
        if model is None:
            self._model = None
            self._check(self._lib.cr_set_vertex_transform(self._ctx, None, 0, None))
            return
        m = (C.c_float * 16)(*[float(x) for x in torch.as_tensor(mvp, dtype=torch.float32).reshape(-1).tolist()])
        self._model = model
        self._check(self._lib.cr_set_vertex_transform(self._ctx, model.data_ptr(), model.stride(0), m))

    def setIndexBuffer(self, buf, ofs: int, numTris: int) -> None:
        self._need_init()
        ptr = _ptr_of(buf)
        self._ib = buf
        self._check(self._lib.cr_set_index_buffer(self._ctx, ptr, int(ofs), int(numTris)))

    def setTuning(self, bin_log2=0, bin_chunk_tris=0, coarse_unit_entries=0, fine_warps=0, fine_ctas_per_sm=0,
                  fine_self_pixels=0):
        self._need_init()
        t = _lib.Tuning(bin_log2, bin_chunk_tris, coarse_unit_entries, fine_warps, fine_ctas_per_sm, fine_self_pixels)
        self._check(self._lib.cr_set_tuning(self._ctx, C.byref(t)))

    def setStageTiming(self, enabled: bool) -> None:
        """Per-stage events for getStats (on by default); off lets the stages' launches overlap."""
        self._need_init()
        self._check(self._lib.cr_set_stage_timing(self._ctx, 1 if enabled else 0))

    def setCapacity(self, max_subtris=0, max_bin_entries=0, max_tile_entries=0):
        self._need_init()
        self._check(self._lib.cr_set_capacity(self._ctx, int(max_subtris), int(max_bin_entries),
                                              int(max_tile_entries)))

    def drawTriangles(self, stream: torch.cuda.Stream | None = None) -> None:
        self._need_init()
        s = (stream or torch.cuda.current_stream()).cuda_stream
        self._check(self._lib.cr_draw_triangles(self._ctx, C.c_void_p(s)))

    def drawTrianglesAsync(self, stream: torch.cuda.Stream | None = None) -> None:
        self._need_init()
        s = (stream or torch.cuda.current_stream()).cuda_stream
        self._check(self._lib.cr_draw_triangles_async(self._ctx, C.c_void_p(s)))

    def _instances(self, instances: list[dict]):
        arr = (_lib.Instance * len(instances))()
        keep = []
        for i, d in enumerate(instances):
            col, dep = d["color"], d["depth"]
            name = d["pipe"].encode()
            keep.append(name)
            clear = d.get("clear")
            arr[i].pipe = name
            arr[i].color = col.getDevicePtr()
            arr[i].depth = dep.getDevicePtr()
            arr[i].width, arr[i].height = col.getSize()
            arr[i].num_samples = col.getNumSamples()
            arr[i].vertices = _ptr_of(d["vertices"])
            arr[i].indices = _ptr_of(d["indices"])
            arr[i].num_tris = int(d["numTris"])
            if clear is not None:
                arr[i].deferred_clear = 1
                arr[i].clear_color = self._lib.cr_color_to_abgr(*[float(c) for c in clear[:4]])
                arr[i].clear_depth = self._lib.cr_clear_depth_from_float(float(clear[4]))
        return arr, keep

    def drawBatch(self, instances: list[dict], stream: torch.cuda.Stream | None = None, sync: bool = True) -> None:
        """Draw several independent scenes in one set of launches. Each dict has
        pipe, color, depth (CudaSurface), vertices, indices (tensor/Buffer),
        numTris and optionally clear=(r, g, b, a, depth)."""
        self._need_init()
        arr, keep = self._instances(instances)
        s = (stream or torch.cuda.current_stream()).cuda_stream
        fn = self._lib.cr_draw_batch if sync else self._lib.cr_draw_batch_async
        self._check(fn(self._ctx, arr, len(instances), C.c_void_p(s)))

    def createBatchGraph(self, instances: list[dict], stream: torch.cuda.Stream | None = None) -> "BatchGraph":
        """Capture the batched draw of `instances` into a CUDA graph (see cr_batch_graph_create)."""
        self._need_init()
        arr, keep = self._instances(instances)
        s = (stream or torch.cuda.current_stream()).cuda_stream
        h = C.c_void_p()
        self._check(self._lib.cr_batch_graph_create(self._ctx, arr, len(instances), C.c_void_p(s), C.byref(h)))
        return BatchGraph(self, h, keep, instances)

    def getStats(self) -> Stats:
        self._need_init()
        s = _lib.Stats()
        self._check(self._lib.cr_get_stats(self._ctx, C.byref(s)))
        return Stats(s.setup_time, s.bin_time, s.coarse_time, s.fine_time)

    def getCounters(self) -> dict:
        self._need_init()
        c = _lib.Counters()
        self._check(self._lib.cr_get_counters(self._ctx, C.byref(c)))
        return {f: getattr(c, f) for f, _ in _lib.Counters._fields_}

    def getProfilingInfo(self) -> str:
        self._need_init()
        buf = C.create_string_buffer(4096)
        self._check(self._lib.cr_get_profiling_info(self._ctx, buf, len(buf)))
        return buf.value.decode()

    def setDebugParams(self, p: DebugParams) -> None:
        self._need_init()
        d = _lib.DebugParams(int(p.emulateTriangleSetup), int(p.emulateBinRaster), int(p.emulateCoarseRaster),
                             int(p.emulateFineRaster))
        self._check(self._lib.cr_set_debug_params(self._ctx, C.byref(d)))


class BatchGraph:
    """A captured batched draw; launch() replays it asynchronously."""

    def __init__(self, raster: CudaRaster, handle, keep, instances):
        self._raster = raster
        self._h = handle
        self._keep = (keep, instances)

    def launch(self, stream: torch.cuda.Stream | None = None) -> None:
        s = (stream or torch.cuda.current_stream()).cuda_stream
        self._raster._check(self._raster._lib.cr_batch_graph_launch(self._h, C.c_void_p(s)))

    def counters(self, stream: torch.cuda.Stream | None = None) -> dict:
        s = (stream or torch.cuda.current_stream()).cuda_stream
        c = _lib.Counters()
        self._raster._check(self._raster._lib.cr_batch_graph_counters(self._h, C.c_void_p(s), C.byref(c)))
        return {f: getattr(c, f) for f, _ in _lib.Counters._fields_}

    def destroy(self) -> None:
        if self._h:
            self._raster._lib.cr_batch_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def _ptr_of(buf) -> int | None:
    if buf is None:
        return None
    if isinstance(buf, Buffer):
        return buf.getCudaPtr()
    if isinstance(buf, torch.Tensor):
        if not buf.is_cuda:
            raise RasterError(1, "CudaRaster: buffers must live in device memory")
        return buf.data_ptr()
    return int(buf)


def vertex_shader_passthrough(model: torch.Tensor, mvp, colors: torch.Tensor | None = None,
                              out: torch.Tensor | None = None, stream: torch.cuda.Stream | None = None) -> torch.Tensor:
    """clip = MVP * (model, 1) on the GPU (the reference's vertexShader_passthrough).
    model: [N, >=3] float32 CUDA tensor; colors: optional [N, 4]; returns [N, 8] (or [N, 4]) records."""
    lib = _lib.load()
    n = model.shape[0]
    width = 8 if colors is not None else 4
    if out is None:
        out = torch.empty((n, width), dtype=torch.float32, device=model.device)
    m = (C.c_float * 16)(*[float(x) for x in torch.as_tensor(mvp, dtype=torch.float32).reshape(-1).tolist()])
    s = (stream or torch.cuda.current_stream()).cuda_stream
    check(lib.cr_vertex_shader_passthrough(model.data_ptr(), model.stride(0), colors.data_ptr() if colors is not None
                                           else None, colors.stride(0) if colors is not None else 0, out.data_ptr(),
                                           width * 4, n, m, C.c_void_p(s)))
    return out


def _vertex_constants(pos_to_clip, pos_to_camera, normal_to_camera):
    k = _lib.VertexConstants()
    for name, m, n in (("pos_to_clip", pos_to_clip, 16), ("pos_to_camera", pos_to_camera, 16),
                       ("normal_to_camera", normal_to_camera, 9)):
        vals = [float(x) for x in torch.as_tensor(m, dtype=torch.float32).reshape(-1).tolist()]
        if len(vals) != n:
            raise RasterError(1, f"{name} needs {n} values")
        getattr(k, name)[:] = vals
    return k


def vertex_shader_gouraud(vertices: torch.Tensor, pos_to_clip, pos_to_camera, normal_to_camera,
                          materials: torch.Tensor, material_idx: torch.Tensor, out: torch.Tensor | None = None,
                          stream: torch.cuda.Stream | None = None) -> torch.Tensor:
    """The reference's vertexShader_gouraud on the GPU. vertices: [N, 8] InputVertex
    records (position, normal, texture coordinate); materials: [M, K] float32 rows, K >= 8,
    starting with diffuse rgba, specular rgb, glossiness (K = 144 for the reference's
    Material records); material_idx: [N] int32. Returns [N, 8] GouraudVertex records
    (clip position, lit colour)."""
    lib = _lib.load()
    n = vertices.shape[0]
    if out is None:
        out = torch.empty((n, 8), dtype=torch.float32, device=vertices.device)
    k = _vertex_constants(pos_to_clip, pos_to_camera, normal_to_camera)
    s = (stream or torch.cuda.current_stream()).cuda_stream
    check(lib.cr_vertex_shader_gouraud(vertices.data_ptr(), n, C.byref(k), materials.data_ptr(),
                                       materials.shape[1] * 4, materials.shape[0], material_idx.data_ptr(),
                                       out.data_ptr(), C.c_void_p(s)))
    return out


def vertex_shader_tex_phong(vertices: torch.Tensor, pos_to_clip, pos_to_camera, normal_to_camera,
                            out: torch.Tensor | None = None, stream: torch.cuda.Stream | None = None) -> torch.Tensor:
    """The reference's vertexShader_texPhong on the GPU: [N, 8] InputVertex records ->
    [N, 16] ShadedVertex_texPhong records."""
    lib = _lib.load()
    n = vertices.shape[0]
    if out is None:
        out = torch.empty((n, 16), dtype=torch.float32, device=vertices.device)
    k = _vertex_constants(pos_to_clip, pos_to_camera, normal_to_camera)
    s = (stream or torch.cuda.current_stream()).cuda_stream
    check(lib.cr_vertex_shader_tex_phong(vertices.data_ptr(), n, C.byref(k), out.data_ptr(), C.c_void_p(s)))
    return out


MATERIAL_FLOATS = 144   # the reference's Material record (Shaders.hpp): 576 bytes


def material_records(diffuse, specular, glossiness, diffuse_texture=None, alpha_texture=None):
    """Packs materials into [M, 144] float32 Material records. diffuse: [M, 4]; specular:
    [M, 3]; glossiness: [M]; *_texture: optional lists of None or (size_xy, mip_levels)
    with mip_levels [L <= 16, 4] rows (scaleX, scaleY, biasX, biasY) into the atlas
    (levels past L repeat the last)."""
    import numpy as np
    d = np.asarray(diffuse, np.float32).reshape(-1, 4)
    m = np.zeros((d.shape[0], MATERIAL_FLOATS), np.float32)
    m[:, 0:4] = d
    m[:, 4:7] = np.asarray(specular, np.float32).reshape(-1, 3)
    m[:, 7] = np.asarray(glossiness, np.float32).reshape(-1)
    for base, texs in ((8, diffuse_texture), (76, alpha_texture)):
        for i, t in enumerate(texs or []):
            if t is None:
                continue
            size, levels = t
            lv = np.asarray(levels, np.float32).reshape(-1, 4)
            m[i, base:base + 2] = size
            for k in range(16):
                m[i, base + 4 + 4 * k: base + 8 + 4 * k] = lv[min(k, lv.shape[0] - 1)]
    return m


def set_tex_phong_constants(materials: torch.Tensor, triangle_material_idx: torch.Tensor, atlas: torch.Tensor,
                            stream: torch.cuda.Stream | None = None) -> None:
    """Inputs of the PixelPipe_texPhong* pipes (the reference's c_constants and
    t_textureAtlas): materials [M, 144] float32 CUDA tensor of Material records, one
    int32 material index per triangle, atlas [H, W] int32/uint32 RGBA8 texels (R in the
    low byte). The tensors must stay alive while draws use them."""
    s = (stream or torch.cuda.current_stream()).cuda_stream
    check(_lib.load().cr_set_tex_phong_constants(materials.data_ptr(), materials.shape[0],
                                                 triangle_material_idx.data_ptr(), triangle_material_idx.numel(),
                                                 atlas.data_ptr(), atlas.shape[1], atlas.shape[0], C.c_void_p(s)))


def texture_sample(atlas: torch.Tensor, uv: torch.Tensor, hardware: bool = False,
                   stream: torch.cuda.Stream | None = None) -> torch.Tensor:
    """The textured pipe's atlas filter at uv [N, 2] (float32 CUDA): [N, 4] channels in
    [0, 1]. hardware=True runs the same lookups through the texture unit instead."""
    out = torch.empty((uv.shape[0], 4), dtype=torch.float32, device=uv.device)
    s = (stream or torch.cuda.current_stream()).cuda_stream
    fn = _lib.load().cr_texture_sample_hw if hardware else _lib.load().cr_texture_sample
    check(fn(atlas.data_ptr(), atlas.shape[1], atlas.shape[0], uv.data_ptr(), out.data_ptr(), uv.shape[0],
             C.c_void_p(s)))
    return out


def pow_exact(x: torch.Tensor, y: torch.Tensor, stream: torch.cuda.Stream | None = None) -> torch.Tensor:
    """The vertex lighting's exact power, elementwise on float32 CUDA tensors."""
    out = torch.empty_like(x)
    s = (stream or torch.cuda.current_stream()).cuda_stream
    check(_lib.load().cr_pow_exact(x.data_ptr(), y.data_ptr(), out.data_ptr(), x.numel(), C.c_void_p(s)))
    return out


def encode_depth(d: int) -> int:
    return _lib.load().cr_encode_depth(d)


def color_to_abgr(r, g, b, a) -> int:
    return _lib.load().cr_color_to_abgr(r, g, b, a)


def clear_depth_from_float(d: float) -> int:
    return _lib.load().cr_clear_depth_from_float(d)


def write_ppm(path, rgba) -> None:
    """Writes an (height, width, 4) uint8 image (e.g. CudaSurface.resolve())
    as a binary PPM (alpha dropped), for looking at frames and diffs."""
    import numpy as np
    a = rgba.cpu().numpy() if hasattr(rgba, "cpu") else np.asarray(rgba)
    a = np.ascontiguousarray(a[..., :3], dtype=np.uint8)
    h, w = a.shape[:2]
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(a.tobytes())
