"""The native library builds for sm_103a, loads, and exports every entry point
that include/cudaraster.h declares; host-only entry points behave without a GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import pkg_mod

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    build = pkg_mod("build")
    build.build_library()
    return pkg_mod("_lib").load()


def declared_entry_points():
    text = (ROOT / "include" / "cudaraster.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cr_[a-z_0-9]+)\s*\(", text)))


def test_header_symbols_exported(lib):
    names = declared_entry_points()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_header():
    binding = set(pkg_mod("_lib").exported_symbols())
    declared = set(declared_entry_points())
    assert binding <= declared


def test_builtin_pipes_registered(lib):
    raster = pkg_mod("raster")
    names = raster.pipe_names()
    for n in ["PixelPipe_gouraud", "PixelPipe_passthrough", "PixelPipe_gouraud_msaa4", "PixelPipe_gouraud_srcover"]:
        assert n in names
    info = raster.pipe_info("PixelPipe_gouraud_msaa4")
    assert info.samples_log2 == 2 and info.vertex_struct_size == 32 and info.render_mode_flags == 3
    assert info.blend_shader_name == b"BlendReplace"
    pt = raster.pipe_info("PixelPipe_passthrough")
    assert pt.vertex_struct_size == 16 and pt.fragment_shader_name == b"FragmentShader_passthrough"


def test_host_helpers_match_reference_host_code(lib):
    """cr_color_to_abgr / cr_encode_depth restate Math.cpp:41-48 and Util.hpp:290-310."""
    import numpy as np
    z = np.load(ROOT / "tests" / "golden" / "ref_shading.npz")
    for c, ref in zip(z["colors"][:2000], z["host_abgr"][:2000]):
        assert lib.cr_color_to_abgr(*map(float, c)) == ref
    m = np.load(ROOT / "tests" / "golden" / "ref_misc.npz")
    for v, e, d in zip(m["depth_in"], m["depth_enc"], m["depth_dec"]):
        assert lib.cr_encode_depth(int(v)) == e
        assert lib.cr_decode_depth(int(v)) == d
    assert lib.cr_clear_depth_from_float(1.0) == lib.cr_encode_depth(0xFFFFFFFF)
    assert lib.cr_clear_depth_from_float(0.0) == lib.cr_encode_depth(0)


def test_oracle_clear_values_match_library(lib):
    """The oracle's clear-value helpers (used where the product library must not be
    loaded, e.g. the CPU baseline) equal the library's host arithmetic."""
    from oracle import oracle as orc
    rng = np.random.default_rng(7)
    for rgba in [(0.2, 0.4, 0.8, 1.0), (0.0, 0.0, 0.0, 0.0), (1.0, 1.0, 1.0, 1.0)] + \
            [tuple(rng.uniform(-0.2, 1.2, 4)) for _ in range(200)]:
        d = float(rgba[0])
        c, z = orc.clear_values(rgba, d)
        assert c == lib.cr_color_to_abgr(*map(float, rgba))
        assert z == lib.cr_clear_depth_from_float(d)


def test_status_strings(lib):
    assert lib.cr_status_string(0) == b"CR_OK"
    assert lib.cr_status_string(5) == b"CR_ERR_CAPACITY"
    assert lib.cr_abi_version() == 1


def test_unknown_pipe_info(lib):
    info = pkg_mod("_lib").PipeInfo()
    assert lib.cr_pipe_info_by_name(b"NoSuchPipe", C.byref(info)) == 3


def test_static_draw_validates_before_touching_gpu(lib):
    """Argument checks of cr_draw_triangles_static run on the host first."""
    fn = lib.cr_draw_triangles_static
    fn.restype = C.c_int
    fn.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                   C.c_int32, C.c_int32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_char_p, C.c_int64]
    err = C.create_string_buffer(256)
    assert fn(b"NoSuchPipe", 16, 16, 8, 8, 1, 16, 16, 1, 1, 0, 0, None, err, 256) == 3
    assert fn(b"PixelPipe_gouraud", 16, 16, 8, 8, 1, 16, 16, 70000, 1, 0, 0, None, err, 256) == 5
    assert b"65536" in err.value
    assert fn(b"PixelPipe_gouraud", 16, 16, 8, 8, 4, 16, 16, 1, 1, 0, 0, None, err, 256) == 4
