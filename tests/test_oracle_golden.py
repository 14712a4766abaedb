"""The CPU oracle against golden vectors produced by the reference's own device
code (compiled for the host by oracle/ref_harness.cpp, see
tests/golden/make_golden.py). No GPU needed."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as orc

GOLD = Path(__file__).resolve().parent / "golden"
P = lambda a: a.ctypes.data


@pytest.fixture(scope="module")
def lib():
    return orc.load()


def _load(name):
    return np.load(GOLD / name)


def _setup_cases():
    z = _load("ref_setup.npz")
    return sorted({k.split("__")[0] for k in z.files})


@pytest.mark.parametrize("case", _setup_cases())
def test_setup_matches_reference(lib, case):
    z = _load("ref_setup.npz")
    w, h, s, f = (int(x) for x in z[f"{case}__params"])
    verts, idx = z[f"{case}__vertices"], z[f"{case}__indices"]
    pipe = orc.make_pipe(w, h, 1 << s, f, stride=32)
    sub, hdr, dat, used = orc.setup(pipe, verts, idx)
    rsub, rhdr, rdat = z[f"{case}__subtris"], z[f"{case}__headers"], z[f"{case}__data"]
    assert used == rhdr.shape[0]
    np.testing.assert_array_equal(sub, rsub)
    # Words the reference leaves unwritten for the flags (PrivateDefs.hpp:40-62, TriangleSetup.inl:181-194).
    mask = np.zeros(16, bool)
    mask[13:16] = True
    if f & orc.DEPTH:
        mask[0:4] = True
    if f & orc.LERP:
        mask[4:13] = True
    else:
        mask[12] = True
    nt = idx.shape[0]
    for t in range(nt):
        k = int(rsub[t])
        if k == 0:
            continue
        slots_r = [t] if k == 1 else [int(rhdr[t, 3]) + i for i in range(k)]
        slots_o = [t] if k == 1 else [int(hdr[t, 3]) + i for i in range(k)]
        for a, b in zip(slots_r, slots_o):
            np.testing.assert_array_equal(hdr[b], rhdr[a], err_msg=f"{case} tri {t} header")
            np.testing.assert_array_equal(dat[b][mask], rdat[a][mask], err_msg=f"{case} tri {t} data")


def test_edge_coverage_matches_reference(lib):
    z = _load("ref_coverage.npz")
    ex = np.array([lib.or_cover8x8_exact(int(a), int(b), int(c), int(d))
                   for a, b, c, d in zip(z["ox"], z["oy"], z["dx"], z["dy"])], np.uint64)
    np.testing.assert_array_equal(ex, z["exact"])
    co = np.array([lib.or_cover8x8_conservative(int(a), int(b), int(c), int(d))
                   for a, b, c, d in zip(z["ox"], z["oy"], z["dx"], z["dy"])], np.uint64)
    np.testing.assert_array_equal(co, z["conservative"])
    ms = np.array([lib.or_cover_msaa(int(s), *map(int, a)) for s, a in zip(z["msaa_s"], z["msaa_args"])], np.uint32)
    np.testing.assert_array_equal(ms, z["msaa"])


def test_triangle_tile_coverage_matches_reference_lut(lib):
    """The reference's LUT rasterizer (cover8x8_exact_fast) on real triangles equals exact coverage."""
    z = _load("ref_coverage.npz")
    for h, (tx, ty), c1, c4 in zip(z["tri_headers"], z["tri_tiles"], z["tri_cov1"], z["tri_cov4"]):
        hh = np.ascontiguousarray(h, np.uint32)
        assert lib.or_triangle_pixel_coverage(P(hh), int(tx), int(ty), 2048, 2048, 0) == int(c1)
        assert lib.or_triangle_pixel_coverage(P(hh), int(tx), int(ty), 2048, 2048, 2) == int(c4)


def test_to_abgr_matches_reference(lib):
    z = _load("ref_shading.npz")
    got = np.array([lib.or_to_abgr(*map(float, c)) for c in z["colors"]], np.uint32)
    np.testing.assert_array_equal(got, z["abgr"])
    got = np.array([lib.or_host_to_abgr(*map(float, c)) for c in z["colors"]], np.uint32)
    np.testing.assert_array_equal(got, z["host_abgr"])


def test_blend_matches_reference(lib):
    z = _load("ref_shading.npz")
    w = C.c_int()
    for m, s, d, out, wr in zip(z["blend_mode"], z["blend_src"], z["blend_dst"], z["blend_out"], z["blend_write"]):
        r = lib.or_blend(int(m), int(s), int(d), C.byref(w))
        assert w.value == wr
        if wr:
            assert r == out


def test_barys_match_reference(lib):
    z = _load("ref_shading.npz")
    for a, s, (sx, sy), ref in zip(z["bary_in"], z["bary_s"], z["bary_xy"], z["bary_out"]):
        a = np.ascontiguousarray(a)
        o = np.zeros(9, np.float32)
        aw, au, av = a[0:3].copy(), a[3:6].copy(), a[6:9].copy()  # kept alive across the call
        lib.or_compute_barys(int(s), P(aw), P(au), P(av), int(sx), int(sy), P(o))
        same = (o.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(o) & np.isnan(ref))
        assert same.all()


def test_centroid_luts_match_reference(lib):
    z = _load("ref_shading.npz")
    for s in range(4):
        lut = np.zeros(256, np.uint8)
        lib.or_centroid_lut(s, P(lut))
        n = 1 << (1 << s)
        np.testing.assert_array_equal(lut[:n], z["centroid_luts"][s][:n])


def test_gouraud_fragments_match_reference(lib):
    z = _load("ref_shading.npz")
    pipe = orc.make_pipe(1024, 768, 1, orc.DEPTH | orc.LERP)
    dat = np.ascontiguousarray(z["cube_data"])
    verts = np.ascontiguousarray(z["cube_vertices"])
    for (t, px, py), col in zip(z["frag_args"], z["frag_color"]):
        d16 = np.ascontiguousarray(dat[t])
        assert lib.or_fragment(C.byref(pipe), P(d16), P(verts), int(t), int(px), int(py), 0x11) == col


def test_depth_codec_flips_perspective_clip_match_reference(lib):
    z = _load("ref_misc.npz")
    for v, e, d in zip(z["depth_in"], z["depth_enc"], z["depth_dec"]):
        assert lib.or_encode_depth(int(v)) == e
        assert lib.or_decode_depth(int(v)) == d
    for (a, b), f in zip(z["flips_in"], z["flips"]):
        assert lib.or_select_flips(int(a), int(b)) == f
    for (fov, n, f), ref in zip(z["persp_args"], z["persp"]):
        o = np.zeros(16, np.float32)
        lib.or_perspective(float(fov), float(n), float(f), P(o))
        np.testing.assert_array_equal(o.view(np.uint32), ref.view(np.uint32))
    for inp, out, n in zip(z["clip_in"], z["clip_out"], z["clip_n"]):
        v = inp[:12].reshape(3, 4)
        b = np.zeros(18, np.float32)
        v0, v1, v2 = v[0].copy(), v[1].copy(), v[2].copy()
        d1, d2 = inp[12:16].copy(), inp[16:20].copy()
        got = lib.or_clip_triangle(P(b), P(v0), P(v1), P(v2), P(d1), P(d2))
        assert got == n
        np.testing.assert_array_equal(b[: 2 * n].view(np.uint32), out[: 2 * n].view(np.uint32))


@pytest.mark.skipif(not orc.ref_available(), reason="reference harness not built (reference sources absent)")
def test_oracle_setup_against_live_reference_random(lib):
    """Where the reference sources are mounted: fresh random clip-heavy scenes, all flag/sample combinations."""
    ref = orc.load_ref()
    rng = np.random.default_rng(12345)
    for s in range(4):
        for f in range(4):
            n = 400
            w = rng.uniform(0.2, 10, n * 3).astype(np.float32)
            c = rng.uniform(-2.5, 2.5, (n, 3))
            ndc = (c[:, None, :] + rng.normal(0, 0.08, (n, 3, 3))).reshape(-1, 3)
            v = np.zeros((n * 3, 8), np.float32)
            v[:, :3] = ndc * w[:, None]
            v[:, 3] = w
            v[:, 4:] = rng.uniform(0, 1, (n * 3, 4))
            idx = np.arange(n * 3, dtype=np.int32).reshape(-1, 3)
            ms = n * 8 + 16
            rsub = np.zeros(n, np.uint8)
            rh = np.zeros((ms, 4), np.uint32)
            rd = np.zeros((ms, 16), np.uint32)
            used = ref.ref_triangle_setup(s, f, 500, 300, 32, P(v), P(idx), n, P(rsub), P(rh), P(rd), ms)
            sub, hdr, dat, oused = orc.setup(orc.make_pipe(500, 300, 1 << s, f), v, idx)
            assert used == oused
            np.testing.assert_array_equal(sub, rsub)


def test_vertex_shaders_match_reference():
    # Shaders.cu:56-108 compiled from the reference's source, powf bound to the specified power.
    from oracle import vertex_oracle as vo
    z = _load("ref_shaders.npz")
    k = [z["pos_to_clip"], z["pos_to_camera"], z["normal_to_camera"]]
    g = vo.vertex_gouraud(z["input"], *k, z["materials"], z["vertex_material_idx"])
    assert np.array_equal(g.view(np.uint32), z["gouraud"].view(np.uint32))
    t = vo.vertex_tex_phong(z["input"], *k)
    assert np.array_equal(t.view(np.uint32), z["tex_phong"].view(np.uint32))


@pytest.mark.parametrize("s", [0, 2])
def test_tex_phong_fragments_match_reference(lib, s):
    # FragmentShader_texPhong::run (Shaders.cu:149-193) from the reference's source, with
    # log2f / powf / tex2D bound to the specified versions; discards included.
    z = _load("ref_shaders.npz")
    orc.set_tex_phong(z["materials"], z["triangle_material_idx"], z["atlas"])
    pipe = orc.make_pipe(320, 240, 1 << s, orc.DEPTH | orc.LERP, "replace", "texphong", 64)
    verts = np.ascontiguousarray(z["tex_phong"])
    dat = z[f"s{s}_data"]
    discards = 0
    for (slot, px, py, cen), col, disc in zip(z[f"s{s}_args"], z[f"s{s}_color"], z[f"s{s}_discard"]):
        d16 = np.ascontiguousarray(dat[slot])
        got = lib.or_fragment(C.byref(pipe), P(d16), P(verts), int(slot), int(px), int(py), int(cen))
        if disc:
            discards += 1
            assert got == 0          # the oracle returns 0 for a discarded fragment
        else:
            assert got == col
    assert 0 < discards < len(z[f"s{s}_color"])
