"""Generates the golden fixtures in this directory from the reference's own
device code, compiled for the host by oracle/Makefile (target `ref`, output
oracle/_ref/libcrref.so; needs the reference sources, named by the
CR_REFERENCE_DIR environment variable, so this script runs where they are
mounted, not on the GPU machine).

    CR_REFERENCE_DIR=<reference checkout> make -C oracle ref && python tests/golden/make_golden.py

Fixtures (npz, seeded inputs + the reference's outputs):
  ref_setup.npz     triangle setup of several scenes (headers, data, subtri counts)
  ref_coverage.npz  8x8 pixel coverage (exact LUT path and conservative), MSAA sample coverage
  ref_shading.npz   toABGR, host toABGR, blends, barycentrics, Gouraud fragments, centroid LUTs
  ref_misc.npz      encodeDepth/decodeDepth, selectFlips, perspective matrices, clipping
  ref_shaders.npz   the example shaders of test/shader/Shaders.cu: Gouraud and texPhong vertex
                    shaders, FragmentShader_texPhong fragments (1 and 4 samples), with log2f /
                    powf / tex2D bound to the pipeline's specified versions (oracle/ref_shaders.cpp)

`python tests/golden/make_golden.py shaders` writes ref_shaders.npz alone.
"""
from __future__ import annotations

import ctypes as C
import importlib
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import oracle as orc  # noqa: E402

scenes = importlib.import_module("cudaraster-linux_gb300.scenes")
P = lambda a: a.ctypes.data


def clip_scene(rng, n, spread, width, height):
    """Small clip-space triangles, a share of them crossing the frustum planes."""
    w = rng.uniform(0.2, 10, size=(n * 3,)).astype(np.float32)
    c = rng.uniform(-spread, spread, size=(n, 3))
    off = rng.normal(0, 0.05, size=(n, 3, 3))
    ndc = (c[:, None, :] + off).reshape(-1, 3)
    v = np.zeros((n * 3, 8), np.float32)
    v[:, 0:3] = ndc * w[:, None]
    v[:, 3] = w
    v[:, 4:8] = rng.uniform(0, 1, size=(n * 3, 4))
    return {"vertices": v, "indices": np.arange(n * 3, dtype=np.int32).reshape(-1, 3), "width": width,
            "height": height}


def run_setup(ref, sc, s, flags, stride=32):
    t = sc["indices"].shape[0]
    ms = t * 8 + 16
    v = np.ascontiguousarray(sc["vertices"][:, : stride // 4], dtype=np.float32)
    i = np.ascontiguousarray(sc["indices"], dtype=np.int32)
    sub = np.zeros(t, np.uint8)
    hdr = np.zeros((ms, 4), np.uint32)
    dat = np.zeros((ms, 16), np.uint32)
    used = ref.ref_triangle_setup(s, flags, sc["width"], sc["height"], stride, P(v), P(i), t, P(sub), P(hdr), P(dat), ms)
    return sub, hdr[:used], dat[:used]


def shaders(ref):
    """Vertex and texPhong fragment shaders of the reference, on the textured heightfield."""
    rng = np.random.default_rng(20261204)
    sc = scenes.textured_terrain(32, 320, 240, seed=3)
    inp = np.ascontiguousarray(sc["input"], np.float32)
    n = inp.shape[0]
    k = [np.ascontiguousarray(sc[x], np.float32) for x in ("pos_to_clip", "pos_to_camera", "normal_to_camera")]
    mats = np.ascontiguousarray(sc["materials"], np.float32)
    vidx = rng.integers(0, mats.shape[0], n).astype(np.int32)
    gouraud = np.zeros((n, 8), np.float32)
    ref.ref_vertex_gouraud(P(inp), n, P(k[0]), P(k[1]), P(k[2]), P(mats), P(vidx), P(gouraud))
    tex_phong = np.zeros((n, 16), np.float32)
    ref.ref_vertex_tex_phong(P(inp), n, P(k[0]), P(k[1]), P(k[2]), P(tex_phong))
    tri = np.ascontiguousarray(sc["triangle_material_idx"], np.int32)
    atlas = np.ascontiguousarray(sc["atlas"], np.uint32)
    ref.ref_set_tex_phong(P(mats), P(tri), P(atlas), atlas.shape[1], atlas.shape[0])
    frag = {}
    for s in (0, 2):
        pipe = orc.make_pipe(320, 240, 1 << s, orc.DEPTH | orc.LERP, "replace", "texphong", 64)
        _, _, dat, used = orc.setup(pipe, tex_phong, sc["indices"])
        m = 2000
        slots = rng.integers(0, used, m)
        args = np.zeros((m, 4), np.int32)   # slot, px, py, centroid
        col = np.zeros(m, np.uint32)
        disc = np.zeros(m, np.int32)
        for j, slot in enumerate(slots):
            d16 = np.ascontiguousarray(dat[slot])
            px, py = int(rng.integers(0, 320)), int(rng.integers(0, 240))
            cen = (int(rng.integers(0, 2 << s)) | (int(rng.integers(0, 2 << s)) << 4)) if s else 0
            dd = C.c_int(0)
            col[j] = ref.ref_tex_phong_fragment(s, P(d16), P(tex_phong), int(slot), px, py, cen, C.byref(dd))
            disc[j] = dd.value
            args[j] = (slot, px, py, cen)
        frag[f"s{s}_data"] = dat[:used]
        frag[f"s{s}_args"] = args
        frag[f"s{s}_color"] = col
        frag[f"s{s}_discard"] = disc
    np.savez_compressed(HERE / "ref_shaders.npz", input=inp, pos_to_clip=k[0], pos_to_camera=k[1],
                        normal_to_camera=k[2], materials=mats, vertex_material_idx=vidx, gouraud=gouraud,
                        tex_phong=tex_phong, triangle_material_idx=tri, atlas=atlas, **frag)


def main():
    if not orc.ref_available():
        sys.exit("oracle/_ref/libcrref.so is missing: run `make -C oracle ref` with CR_REFERENCE_DIR set to the reference sources")
    ref = orc.load_ref()
    if sys.argv[1:] == ["shaders"]:
        shaders(ref)
        print("ref_shaders.npz written to", HERE)
        return
    rng = np.random.default_rng(20261203)

    # ---- setup
    cases = []
    cube = scenes.cube(1024, 768)
    cases.append(("cube_s0_f3", cube, 0, 3))
    cases.append(("cube_s2_f3", cube, 2, 3))
    soup = scenes.soup(3000, 320, 240, seed=7, median_px=6.0)
    for s, f in [(0, 3), (0, 1), (1, 3), (3, 2), (2, 0)]:
        cases.append((f"soup_s{s}_f{f}", soup, s, f))
    for k, spread in enumerate([1.5, 3.0]):
        sc = clip_scene(rng, 1500, spread, 640, 480)
        cases.append((f"clip{k}_s0_f3", sc, 0, 3))
        cases.append((f"clip{k}_s2_f3", sc, 2, 3))
    big = scenes.soup(2000, 2048, 2048, seed=9, median_px=300.0, sigma=1.5)
    cases.append(("guard_s0_f3", big, 0, 3))
    out = {}
    for name, sc, s, f in cases:
        sub, hdr, dat = run_setup(ref, sc, s, f)
        out[f"{name}__vertices"] = sc["vertices"]
        out[f"{name}__indices"] = sc["indices"]
        out[f"{name}__params"] = np.array([sc["width"], sc["height"], s, f], np.int32)
        out[f"{name}__subtris"] = sub
        out[f"{name}__headers"] = hdr
        out[f"{name}__data"] = dat
    np.savez_compressed(HERE / "ref_setup.npz", **out)

    # ---- coverage: random edges (exact + LUT-fast + conservative) and triangle/tile pairs
    n = 20000
    scale = rng.choice([4, 64, 1024, 16384, 32767], size=n)
    dx = (rng.uniform(-1, 1, n) * scale).astype(np.int32)
    dy = (rng.uniform(-1, 1, n) * scale).astype(np.int32)
    near = rng.random(n) < 0.7
    ox = np.where(near, rng.integers(-300, 300, n), rng.integers(-30000, 30000, n)).astype(np.int32)
    oy = np.where(near, rng.integers(-300, 300, n), rng.integers(-30000, 30000, n)).astype(np.int32)
    keep = ~((dx == 0) & (dy == 0))
    dx, dy, ox, oy = dx[keep], dy[keep], ox[keep], oy[keep]
    exact = np.array([ref.ref_cover8x8_exact_ref(int(a), int(b), int(c), int(d)) for a, b, c, d in zip(ox, oy, dx, dy)],
                     np.uint64)
    cons = np.array([ref.ref_cover8x8_conservative_ref(int(a), int(b), int(c), int(d)) for a, b, c, d in
                     zip(ox, oy, dx, dy)], np.uint64)
    ms = rng.integers(1, 4, dx.size).astype(np.int32)
    so = rng.integers(-60, 60, (dx.size, 4)).astype(np.int32)
    msaa = np.array([ref.ref_coverMSAA_ref(int(s), int(a), int(b), int(c), int(d)) for s, (a, b, c, d) in zip(ms, so)],
                    np.uint32)
    # triangles with their tiles, viewport 2048 (the reference's maximum)
    tri_hdr, tri_tile, tri_cov1, tri_cov4 = [], [], [], []
    big_sc = scenes.soup(600, 2048, 2048, seed=3, median_px=120.0, sigma=1.2)
    sub, hdr, _ = run_setup(ref, big_sc, 0, 1)
    for t in range(big_sc["indices"].shape[0]):
        if sub[t] != 1:
            continue
        h = hdr[t]
        xs = [int(np.int16(h[k] & 0xFFFF)) for k in range(3)]
        ys = [int(np.int16(h[k] >> 16)) for k in range(3)]
        tx0, tx1 = max((min(xs) + 2048 * 8) >> 7, 0), min((max(xs) + 2048 * 8) >> 7, 255)
        ty0, ty1 = max((min(ys) + 2048 * 8) >> 7, 0), min((max(ys) + 2048 * 8) >> 7, 255)
        if tx0 > tx1 or ty0 > ty1:
            continue
        for _ in range(4):
            tx, ty = int(rng.integers(tx0, tx1 + 1)), int(rng.integers(ty0, ty1 + 1))
            hh = np.ascontiguousarray(h, np.uint32)
            tri_hdr.append(hh)
            tri_tile.append((tx, ty))
            tri_cov1.append(ref.ref_triangle_pixel_coverage(0, P(hh), tx, ty, 2048, 2048))
            tri_cov4.append(ref.ref_triangle_pixel_coverage(2, P(hh), tx, ty, 2048, 2048))
    np.savez_compressed(HERE / "ref_coverage.npz", ox=ox, oy=oy, dx=dx, dy=dy, exact=exact, conservative=cons,
                        msaa_s=ms, msaa_args=so, msaa=msaa, tri_headers=np.array(tri_hdr, np.uint32),
                        tri_tiles=np.array(tri_tile, np.int32), tri_cov1=np.array(tri_cov1, np.uint64),
                        tri_cov4=np.array(tri_cov4, np.uint64))

    # ---- shading
    cols = np.concatenate([rng.uniform(-0.2, 1.2, (4000, 4)).astype(np.float32),
                           np.array([[0, 1, 0.5 / 255, 1.5 / 255], [np.nan, np.inf, -np.inf, -0.0],
                                     [1e-40, 2.0, 256 / 255, 255.5 / 255]], np.float32)])
    half = ((np.arange(256) + 0.5) / 255).astype(np.float32)
    cols = np.concatenate([cols, np.stack([half, np.nextafter(half, np.float32(2)),
                                           np.nextafter(half, np.float32(-2)), half], axis=1)])
    abgr = np.array([ref.ref_to_abgr(*map(float, c)) for c in cols], np.uint32)
    host_abgr = np.array([ref.ref_host_to_abgr(*map(float, c)) for c in cols], np.uint32)
    bsrc = rng.integers(0, 2**32, 6000, dtype=np.uint64).astype(np.uint32)
    bdst = rng.integers(0, 2**32, 6000, dtype=np.uint64).astype(np.uint32)
    bmode = rng.integers(0, 4, 6000).astype(np.int32)
    w = C.c_int()
    bres, bwrite = [], []
    for m, s_, d_ in zip(bmode, bsrc, bdst):
        bres.append(ref.ref_blend(int(m), int(s_), int(d_), C.byref(w)))
        bwrite.append(w.value)
    nb = 6000
    bary_in = rng.integers(-2**31, 2**31, (nb, 9), dtype=np.int64).astype(np.int32)
    bary_s = rng.integers(0, 4, nb).astype(np.int32)
    bary_xy = rng.integers(0, 4096, (nb, 2)).astype(np.int32)
    bary_out = np.zeros((nb, 9), np.float32)
    for k in range(nb):
        o = np.zeros(9, np.float32)
        a = np.ascontiguousarray(bary_in[k])
        aw, au, av = a[0:3].copy(), a[3:6].copy(), a[6:9].copy()  # kept alive across the call
        ref.ref_compute_barys(int(bary_s[k]), P(aw), P(au), P(av),
                              int(bary_xy[k, 0]), int(bary_xy[k, 1]), P(o))
        bary_out[k] = o
    luts = np.zeros((4, 256), np.uint8)
    for s in range(4):
        lut = np.zeros(256, np.uint8)
        ref.ref_centroid_lut(s, P(lut))
        luts[s] = lut
    # Gouraud fragments of the cube at covered pixels
    sub, hdr, dat = run_setup(ref, cube, 0, 3)
    frag_args, frag_col = [], []
    dat_c = np.ascontiguousarray(dat, np.uint32)
    verts = np.ascontiguousarray(cube["vertices"], np.float32)
    for t in range(cube["indices"].shape[0]):
        if sub[t] != 1:
            continue
        for _ in range(50):
            px, py = int(rng.integers(0, 1024)), int(rng.integers(0, 768))
            frag_args.append((t, px, py))
            frag_col.append(ref.ref_gouraud_fragment(0, 3, P(dat_c), P(verts), t, t, px, py, 0x11))
    np.savez_compressed(HERE / "ref_shading.npz", colors=cols, abgr=abgr, host_abgr=host_abgr, blend_mode=bmode,
                        blend_src=bsrc, blend_dst=bdst, blend_out=np.array(bres, np.uint32),
                        blend_write=np.array(bwrite, np.int32), bary_in=bary_in, bary_s=bary_s, bary_xy=bary_xy,
                        bary_out=bary_out, centroid_luts=luts, cube_data=dat_c, cube_vertices=verts,
                        frag_args=np.array(frag_args, np.int32), frag_color=np.array(frag_col, np.uint32))

    # ---- misc
    dvals = np.concatenate([rng.integers(0, 2**32, 4000, dtype=np.uint64),
                            np.array([0, 1, 2**32 - 1, 2**31, 17600, 2**32 - 17601], np.uint64)]).astype(np.uint32)
    enc = np.array([ref.ref_encode_depth(int(v)) for v in dvals], np.uint32)
    dec = np.array([ref.ref_decode_depth(int(v)) for v in dvals], np.uint32)
    fl = rng.integers(-40000, 40000, (4000, 2)).astype(np.int32)
    fl[:100] = rng.integers(-2, 3, (100, 2))
    flips = np.array([ref.ref_select_flips(int(a), int(b)) for a, b in fl], np.uint32)
    persp_args = np.array([[60, 0.1, 100], [45, 1, 1000], [90, 0.01, 10], [30, 0.5, 50]], np.float32)
    persp = np.zeros((len(persp_args), 16), np.float32)
    for k, (fov, nn, ff) in enumerate(persp_args):
        o = np.zeros(16, np.float32)
        ref.ref_perspective(float(fov), float(nn), float(ff), P(o))
        persp[k] = o
    nclip = 3000
    clip_in = np.zeros((nclip, 20), np.float32)
    clip_out = np.zeros((nclip, 18), np.float32)
    clip_n = np.zeros(nclip, np.int32)
    for k in range(nclip):
        v = rng.normal(0, 1.5, (3, 4)).astype(np.float32)
        v[:, 3] = np.abs(v[:, 3]) + 0.1
        d1 = (v[1] - v[0]).astype(np.float32)
        d2 = (v[2] - v[0]).astype(np.float32)
        b = np.zeros(18, np.float32)
        v0, v1, v2 = v[0].copy(), v[1].copy(), v[2].copy()  # kept alive across the call
        clip_n[k] = ref.ref_clip_triangle(P(b), P(v0), P(v1), P(v2), P(d1), P(d2))
        clip_in[k] = np.concatenate([v.reshape(-1), d1, d2])[:20]
        clip_out[k] = b
    np.savez_compressed(HERE / "ref_misc.npz", depth_in=dvals, depth_enc=enc, depth_dec=dec, flips_in=fl,
                        flips=flips, persp_args=persp_args, persp=persp, clip_in=clip_in, clip_out=clip_out,
                        clip_n=clip_n)
    shaders(ref)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
