"""ctypes wrapper of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker. The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libcrref.so"

DEPTH, LERP, QUADS = 1, 2, 4
BLENDS = {"replace": 0, "srcover": 1, "additive": 2, "depthonly": 3}
SHADERS = {"gouraud": 0, "red": 1, "trihash": 2, "deriv": 3, "texphong": 4}


class Pipe(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("samples_log2", C.c_int32),
                ("render_mode", C.c_uint32), ("blend", C.c_int32), ("shader", C.c_int32),
                ("vertex_stride", C.c_int32), ("deferred_clear", C.c_int32), ("clear_color", C.c_uint32),
                ("clear_depth", C.c_uint32)]


class OrStats(C.Structure):
    _fields_ = [("num_subtris", C.c_int64), ("num_clipped", C.c_int64), ("num_fragments", C.c_int64),
                ("zmin_violations", C.c_int64), ("tile_entries", C.c_int64)]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            subprocess.run(["make", "-C", str(HERE), "liboracle.so"], check=True, capture_output=True)
        lib = C.CDLL(str(LIB))
        lib.or_setup.restype = C.c_int64
        lib.or_setup.argtypes = [C.POINTER(Pipe), C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_int64]
        lib.or_render.restype = C.c_int
        lib.or_render.argtypes = [C.POINTER(Pipe), C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                  C.c_int, C.POINTER(OrStats)]
        for name, res, args in [
            ("or_to_abgr", C.c_uint32, [C.c_float] * 4), ("or_host_to_abgr", C.c_uint32, [C.c_float] * 4),
            ("or_encode_depth", C.c_uint32, [C.c_uint32]), ("or_decode_depth", C.c_uint32, [C.c_uint32]),
            ("or_clear_depth", C.c_uint32, [C.c_float]),
            ("or_blend", C.c_uint32, [C.c_int, C.c_uint32, C.c_uint32, C.POINTER(C.c_int)]),
            ("or_select_flips", C.c_uint32, [C.c_int32, C.c_int32]),
            ("or_select_msaa_centroid", C.c_int, [C.c_int, C.c_uint32]),
            ("or_centroid_lut", None, [C.c_int, C.c_void_p]),
            ("or_setup_pleq", None, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_int, C.c_void_p]),
            ("or_clip_triangle", C.c_int, [C.c_void_p] * 6),
            ("or_cover8x8_exact", C.c_uint64, [C.c_int32] * 4),
            ("or_cover8x8_conservative", C.c_uint64, [C.c_int32] * 4),
            ("or_cover_msaa", C.c_uint32, [C.c_int] + [C.c_int32] * 4),
            ("or_triangle_pixel_coverage", C.c_uint64, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
            ("or_triangle_sample_coverage", C.c_uint32, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
            ("or_compute_barys", None, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
            ("or_find_bit", C.c_int, [C.c_uint64, C.c_int, C.c_int]),
            ("or_fragment", C.c_uint32, [C.POINTER(Pipe), C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                         C.c_uint32]),
            ("or_perspective", None, [C.c_float, C.c_float, C.c_float, C.c_void_p]),
            ("or_f32_to_s32_sat", C.c_int32, [C.c_float]), ("or_f32_to_u32_sat", C.c_uint32, [C.c_float]),
            ("or_f32_to_u32_sat_rmi", C.c_uint32, [C.c_float]), ("or_f32_to_s64", C.c_int64, [C.c_float]),
            ("or_f32_to_u32_rz", C.c_uint32, [C.c_float]),
            ("or_set_tex_phong", None, [C.c_void_p, C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_int, C.c_int]),
            ("or_texture_sample", None, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int64]),
            ("or_pow_exact", C.c_float, [C.c_float, C.c_float]),
            ("or_tex_normalize_mismatches", C.c_int64, []),
            ("or_log2_exact", C.c_float, [C.c_float]),
            ("or_evaluate_lighting", None, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p]),
            ("or_queue_lists", C.c_int64, [C.POINTER(Pipe), C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int,
                                           C.c_void_p, C.c_void_p, C.c_int64]),
        ]:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def make_pipe(width, height, samples=1, flags=DEPTH | LERP, blend="replace", shader="gouraud", stride=32,
              clear=None) -> Pipe:
    p = Pipe()
    p.width, p.height = width, height
    p.samples_log2 = int(samples).bit_length() - 1
    p.render_mode = flags
    p.blend = BLENDS[blend]
    p.shader = SHADERS[shader]
    p.vertex_stride = stride
    if clear is not None:
        p.deferred_clear = 1
        p.clear_color, p.clear_depth = clear
    return p


def clear_values(rgba=(0.2, 0.4, 0.8, 1.0), depth=1.0):
    """(ABGR8 colour, encoded depth) of a deferred clear, by the oracle's restatement of the
    reference's host arithmetic (Math.cpp:41-48, CudaRaster.cpp:174-179)."""
    lib = load()
    return int(lib.or_host_to_abgr(*[float(c) for c in rgba])), int(lib.or_clear_depth(float(depth)))


def surface_shape(width, height, samples):
    return ((height + 7) & ~7, ((width + 7) & ~7) * samples)


def render(pipe: Pipe, vertices: np.ndarray, indices: np.ndarray, color=None, depth=None, threads: int = 0):
    """Renders in place into color/depth (uint32 arrays of surface_shape), returns (color, depth, stats)."""
    lib = load()
    shape = surface_shape(pipe.width, pipe.height, 1 << pipe.samples_log2)
    color = np.zeros(shape, np.uint32) if color is None else np.ascontiguousarray(color, dtype=np.uint32)
    depth = np.zeros(shape, np.uint32) if depth is None else np.ascontiguousarray(depth, dtype=np.uint32)
    v = np.ascontiguousarray(vertices, dtype=np.float32)
    i = np.ascontiguousarray(indices, dtype=np.int32)
    st = OrStats()
    lib.or_render(C.byref(pipe), v.ctypes.data, i.ctypes.data, i.shape[0], color.ctypes.data, depth.ctypes.data,
                  int(threads), C.byref(st))
    return color, depth, {f: getattr(st, f) for f, _ in OrStats._fields_}


def setup(pipe: Pipe, vertices: np.ndarray, indices: np.ndarray, max_subtris: int | None = None):
    """Triangle setup outputs: (tri_subtris[T], headers[S,4], data[S,16], used)."""
    lib = load()
    v = np.ascontiguousarray(vertices, dtype=np.float32)
    i = np.ascontiguousarray(indices, dtype=np.int32)
    t = i.shape[0]
    ms = max_subtris or (t * 7 + 16)
    sub = np.zeros(t, np.uint8)
    hdr = np.zeros((ms, 4), np.uint32)
    dat = np.zeros((ms, 16), np.uint32)
    used = lib.or_setup(C.byref(pipe), v.ctypes.data, i.ctypes.data, t, sub.ctypes.data, hdr.ctypes.data,
                        dat.ctypes.data, ms)
    return sub, hdr, dat, used


QUEUE_KINDS = {"bin_exact": 0, "bin_rule": 1, "tile_exact": 2, "tile_rule": 3}


def queue_lists(pipe: Pipe, vertices: np.ndarray, indices: np.ndarray, bin_log2: int, kind: str):
    """Per-cell bin or tile lists of a draw as (offsets [cells + 1], entries) int64 / uint32
    arrays (cells in row-major order): "bin_exact" / "tile_exact" hold the entries that
    cover a sample of the cell, "bin_rule" / "tile_rule" those the GPU binning rule keeps."""
    lib = load()
    v = np.ascontiguousarray(vertices, dtype=np.float32)
    i = np.ascontiguousarray(indices, dtype=np.int32)
    k = QUEUE_KINDS[kind]
    total = lib.or_queue_lists(C.byref(pipe), v.ctypes.data, i.ctypes.data, i.shape[0], bin_log2, k, None, None, 0)
    if total < 0:
        raise ValueError("bad queue-list arguments")
    wt, ht = (pipe.width + 7) >> 3, (pipe.height + 7) >> 3
    side = 1 << bin_log2
    cells = ((wt + side - 1) // side) * ((ht + side - 1) // side) if k < 2 else wt * ht
    off = np.zeros(cells + 1, np.int64)
    ent = np.zeros(max(total, 1), np.uint32)
    lib.or_queue_lists(C.byref(pipe), v.ctypes.data, i.ctypes.data, i.shape[0], bin_log2, k, off.ctypes.data,
                       ent.ctypes.data, total)
    return off, ent[:total]


_tex_phong_keep = None


def set_tex_phong(materials: np.ndarray, triangle_material_idx: np.ndarray, atlas: np.ndarray) -> None:
    """Inputs of the textured Phong shader: materials [M, 144] float32 (576-byte Material
    records), one int32 material index per triangle, an RGBA8 atlas [H, W] uint32."""
    global _tex_phong_keep
    lib = load()
    m = np.ascontiguousarray(materials, dtype=np.float32).reshape(-1, 144)
    t = np.ascontiguousarray(triangle_material_idx, dtype=np.int32).reshape(-1)
    a = np.ascontiguousarray(atlas, dtype=np.uint32)
    _tex_phong_keep = (m, t, a)
    lib.or_set_tex_phong(m.ctypes.data, m.shape[0], t.ctypes.data, t.shape[0], a.ctypes.data, a.shape[1], a.shape[0])


def texture_sample(atlas: np.ndarray, uv: np.ndarray) -> np.ndarray:
    """The atlas filter at uv [N, 2]: [N, 4] float32 channels."""
    lib = load()
    a = np.ascontiguousarray(atlas, dtype=np.uint32)
    p = np.ascontiguousarray(uv, dtype=np.float32).reshape(-1, 2)
    out = np.zeros((p.shape[0], 4), np.float32)
    lib.or_texture_sample(a.ctypes.data, a.shape[1], a.shape[0], p.ctypes.data, out.ctypes.data, p.shape[0])
    return out


def pow_exact(x: float, y: float) -> float:
    return load().or_pow_exact(x, y)


def log2_exact(x: float) -> float:
    return load().or_log2_exact(x)


def evaluate_lighting(camera_pos, camera_normal, specular, glossiness, diffuse) -> np.ndarray:
    arrs = [np.ascontiguousarray(v, dtype=np.float32) for v in (camera_pos, camera_normal, specular, diffuse)]
    out = np.zeros(3, np.float32)
    load().or_evaluate_lighting(arrs[0].ctypes.data, arrs[1].ctypes.data, arrs[2].ctypes.data, float(glossiness),
                                arrs[3].ctypes.data, out.ctypes.data)
    return out


def ref_available() -> bool:
    return REF_LIB.exists()


def load_ref():
    """The reference's own device code compiled for the host (oracle/_ref, built only where the
    reference sources exist)."""
    lib = C.CDLL(str(REF_LIB))
    lib.ref_triangle_setup.restype = C.c_int
    lib.ref_triangle_setup.argtypes = [C.c_int, C.c_uint, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                       C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    for n in ["ref_cover8x8_exact_ref", "ref_cover8x8_exact_fast", "ref_cover8x8_conservative_ref",
              "ref_cover8x8_conservative_fast", "ref_cover8x8_exact_noLUT", "ref_triangle_pixel_coverage"]:
        getattr(lib, n).restype = C.c_ulonglong
    lib.ref_triangle_pixel_coverage.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
    lib.ref_triangle_sample_coverage.restype = C.c_uint
    lib.ref_triangle_sample_coverage.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
    for n in ["ref_to_abgr", "ref_host_to_abgr"]:
        getattr(lib, n).restype = C.c_uint
        getattr(lib, n).argtypes = [C.c_float] * 4
    for n in ["ref_encode_depth", "ref_decode_depth", "ref_select_flips", "ref_blend", "ref_coverMSAA_ref",
              "ref_coverMSAA_fast", "ref_gouraud_fragment"]:
        getattr(lib, n).restype = C.c_uint
    lib.ref_gouraud_fragment.argtypes = [C.c_int, C.c_uint, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_uint]
    lib.ref_setup_pleq.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_int, C.c_void_p]
    lib.ref_perspective.argtypes = [C.c_float, C.c_float, C.c_float, C.c_void_p]
    lib.ref_compute_barys.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    lib.ref_centroid_lut.argtypes = [C.c_int, C.c_void_p]
    lib.ref_clip_triangle.restype = C.c_int
    lib.ref_clip_triangle.argtypes = [C.c_void_p] * 6
    lib.ref_blend.argtypes = [C.c_int, C.c_uint, C.c_uint, C.POINTER(C.c_int)]
    for n in ["ref_cover8x8_exact_ref", "ref_cover8x8_exact_fast", "ref_cover8x8_conservative_ref",
              "ref_cover8x8_conservative_fast", "ref_cover8x8_exact_noLUT"]:
        getattr(lib, n).argtypes = [C.c_int] * 4
    lib.ref_coverMSAA_ref.argtypes = [C.c_int] * 5
    lib.ref_coverMSAA_fast.argtypes = [C.c_int] * 5
    lib.ref_encode_depth.argtypes = [C.c_uint]
    lib.ref_decode_depth.argtypes = [C.c_uint]
    lib.ref_select_flips.argtypes = [C.c_int, C.c_int]
    lib.ref_vertex_gouraud.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 6
    lib.ref_vertex_tex_phong.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 4
    lib.ref_set_tex_phong.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    lib.ref_tex_phong_fragment.restype = C.c_uint
    lib.ref_tex_phong_fragment.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_uint,
                                           C.POINTER(C.c_int)]
    return lib
