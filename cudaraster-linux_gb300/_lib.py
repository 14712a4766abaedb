"""ctypes binding of the C ABI in include/cudaraster.h.

The shared library is loaded from this package directory only (built by
build.py / __graft_entry__.build()); there is no fallback implementation, so a
missing library is an error.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libcudaraster_gb300.so"

CR_OK = 0
STATUS_NAMES = {
    0: "CR_OK", 1: "CR_ERR_INVALID_ARGUMENT", 2: "CR_ERR_INVALID_STATE", 3: "CR_ERR_NO_PIPE",
    4: "CR_ERR_PIPE_MISMATCH", 5: "CR_ERR_CAPACITY", 6: "CR_ERR_CUDA", 7: "CR_ERR_TIMEOUT",
    8: "CR_ERR_OUT_OF_MEMORY", 9: "CR_ERR_UNSUPPORTED",
}

RENDER_DEPTH = 1
RENDER_LERP = 2
RENDER_QUADS = 4


class Stats(C.Structure):
    _fields_ = [("setup_time", C.c_float), ("bin_time", C.c_float), ("coarse_time", C.c_float),
                ("fine_time", C.c_float)]


class Counters(C.Structure):
    _fields_ = [("num_tris", C.c_int64), ("num_subtris", C.c_int64), ("bin_entries", C.c_int64),
                ("tile_entries", C.c_int64), ("coarse_units", C.c_int64), ("max_subtris", C.c_int64),
                ("max_bin_entries", C.c_int64), ("max_tile_entries", C.c_int64), ("reruns", C.c_int32),
                ("overflow", C.c_int32), ("num_bins", C.c_int32), ("num_tiles", C.c_int32)]


class PipeInfo(C.Structure):
    _fields_ = [("name", C.c_char * 64), ("samples_log2", C.c_int32), ("vertex_struct_size", C.c_int32),
                ("render_mode_flags", C.c_uint32), ("profiling_mode", C.c_int32),
                ("blend_shader_name", C.c_char * 64), ("fragment_shader_name", C.c_char * 64)]


class DebugParams(C.Structure):
    _fields_ = [("emulate_triangle_setup", C.c_int32), ("emulate_bin_raster", C.c_int32),
                ("emulate_coarse_raster", C.c_int32), ("emulate_fine_raster", C.c_int32)]


class Tuning(C.Structure):
    _fields_ = [("bin_log2", C.c_int32), ("bin_chunk_tris", C.c_int32), ("coarse_unit_entries", C.c_int32),
                ("fine_warps", C.c_int32), ("fine_ctas_per_sm", C.c_int32),
                ("fine_self_pixels", C.c_int32)]


class Instance(C.Structure):
    _fields_ = [("pipe", C.c_char_p), ("color", C.c_void_p), ("depth", C.c_void_p), ("width", C.c_int32),
                ("height", C.c_int32), ("num_samples", C.c_int32), ("vertices", C.c_void_p),
                ("indices", C.c_void_p), ("num_tris", C.c_int32), ("deferred_clear", C.c_int32),
                ("clear_color", C.c_uint32), ("clear_depth", C.c_uint32)]


class VertexConstants(C.Structure):
    _fields_ = [("pos_to_clip", C.c_float * 16), ("pos_to_camera", C.c_float * 16), ("normal_to_camera", C.c_float * 9)]


class QueueLayout(C.Structure):
    _fields_ = [("bins_x", C.c_int32), ("bins_y", C.c_int32), ("tiles_x", C.c_int32), ("tiles_y", C.c_int32),
                ("bin_log2", C.c_int32), ("num_bins", C.c_int32), ("num_tiles", C.c_int32),
                ("num_instances", C.c_int32)]


# name -> (restype, argtypes)
_SIGNATURES = {
    "cr_abi_version": (C.c_int32, []),
    "cr_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "cr_destroy": (C.c_int, [C.c_void_p]),
    "cr_status_string": (C.c_char_p, [C.c_int]),
    "cr_last_error": (C.c_char_p, [C.c_void_p]),
    "cr_set_surfaces": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "cr_deferred_clear": (C.c_int, [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float]),
    "cr_deferred_clear_raw": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "cr_set_pixel_pipe": (C.c_int, [C.c_void_p, C.c_char_p]),
    "cr_set_vertex_buffer": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "cr_set_vertex_transform": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "cr_read_setup_output": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "cr_read_queue_output": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int64)]),
    "cr_set_index_buffer": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32]),
    "cr_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "cr_set_debug_params": (C.c_int, [C.c_void_p, C.POINTER(DebugParams)]),
    "cr_set_capacity": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64]),
    "cr_set_stage_timing": (C.c_int, [C.c_void_p, C.c_int32]),
    "cr_draw_triangles": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cr_draw_triangles_async": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cr_draw_batch": (C.c_int, [C.c_void_p, C.POINTER(Instance), C.c_int32, C.c_void_p]),
    "cr_draw_batch_async": (C.c_int, [C.c_void_p, C.POINTER(Instance), C.c_int32, C.c_void_p]),
    "cr_batch_graph_create": (C.c_int, [C.c_void_p, C.POINTER(Instance), C.c_int32, C.c_void_p,
                                        C.POINTER(C.c_void_p)]),
    "cr_batch_graph_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cr_batch_graph_counters": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Counters)]),
    "cr_batch_graph_destroy": (C.c_int, [C.c_void_p]),
    "cr_draw_triangles_static": (C.c_int, [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                           C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_uint32, C.c_uint32,
                                           C.c_void_p, C.c_char_p, C.c_int64]),
    "cr_vertex_shader_passthrough": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                               C.c_int64, C.POINTER(C.c_float), C.c_void_p]),
    "cr_vertex_shader_gouraud": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(VertexConstants), C.c_void_p, C.c_int32,
                                           C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cr_set_tex_phong_constants": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32,
                                             C.c_int32, C.c_void_p]),
    "cr_texture_sample": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "cr_texture_sample_hw": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64,
                                       C.c_void_p]),
    "cr_vertex_shader_tex_phong": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(VertexConstants), C.c_void_p,
                                             C.c_void_p]),
    "cr_pow_exact": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "cr_resolve_color": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p]),
    "cr_get_queue_layout": (C.c_int, [C.c_void_p, C.POINTER(QueueLayout)]),
    "cr_queue_counts": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "cr_queue_features": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_float), C.c_void_p, C.c_void_p]),
    "cr_queue_log_counts": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                      C.c_void_p, C.c_void_p]),
    "cr_queue_targets": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p,
                                   C.c_void_p]),
    "cr_queue_plan": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                C.c_void_p]),
    "cr_predictor_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "cr_predictor_destroy": (None, [C.c_void_p]),
    "cr_predictor_num_params": (C.c_int64, [C.c_void_p]),
    "cr_predictor_steps": (C.c_int64, [C.c_void_p]),
    "cr_predictor_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int64]),
    "cr_predictor_get_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int64]),
    "cr_predictor_get_params_bf16": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint16), C.c_int64]),
    "cr_predictor_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "cr_predictor_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                         C.c_void_p, C.c_void_p, C.c_void_p]),
    "cr_predictor_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                          C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p, C.c_void_p]),
    "cr_predictor_bad_rows": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_int32]),
    "cr_predictor_set_loss_weights": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int64]),
    "cr_predictor_frame": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(QueueLayout),
                                     C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.POINTER(C.c_float), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cr_get_queue_buffers": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                       C.POINTER(C.c_void_p)]),
    "cr_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "cr_get_counters": (C.c_int, [C.c_void_p, C.POINTER(Counters)]),
    "cr_get_profiling_info": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int64]),
    "cr_pipe_count": (C.c_int32, []),
    "cr_pipe_info_at": (C.c_int, [C.c_int32, C.POINTER(PipeInfo)]),
    "cr_pipe_info_by_name": (C.c_int, [C.c_char_p, C.POINTER(PipeInfo)]),
    "cr_color_to_abgr": (C.c_uint32, [C.c_float, C.c_float, C.c_float, C.c_float]),
    "cr_encode_depth": (C.c_uint32, [C.c_uint32]),
    "cr_decode_depth": (C.c_uint32, [C.c_uint32]),
    "cr_clear_depth_from_float": (C.c_uint32, [C.c_float]),
}

_lib = None


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def load(path: Path | None = None):
    """Load the native library (once). Raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: run build() (python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class RasterError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def check(status: int, ctx=None) -> None:
    if status != CR_OK:
        lib = load()
        msg = lib.cr_last_error(ctx).decode() if ctx else ""
        raise RasterError(status, msg or STATUS_NAMES.get(status, "error"))
