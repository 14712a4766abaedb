"""Seeded synthetic scenes for the benchmark configurations and the tests.

Every scene is a dict with clip-space GouraudVertex records (float32 [N, 8]:
clipPos xyzw + RGBA colour in [0, 1]), int32 triangle indices [T, 3] and the
surface description. Vertex positions are produced on the host in float64 and
rounded once to float32, so the rasterizer and the oracle read identical bits.

  cube      -- the reference demo's 12-triangle cube (test/App.cpp:208-230)
  soup      -- random triangle soup (lognormal edge length, 50% back-facing)
  terrain   -- value-noise heightfield grid seen at a grazing angle
  batch     -- many soups with uneven triangle counts and resolutions
"""
from __future__ import annotations

import math

import numpy as np

# test/App.cpp:210-230
CUBE_POSITIONS = np.array([
    [-1, -1, -1], [-1, -1, +1], [-1, +1, -1], [-1, +1, +1],
    [+1, -1, -1], [+1, -1, +1], [+1, +1, -1], [+1, +1, +1]], dtype=np.float64)
CUBE_INDICES = np.array([
    7, 3, 1, 7, 1, 5,
    7, 5, 6, 6, 5, 4,
    6, 4, 2, 2, 4, 0,
    2, 0, 3, 3, 0, 1,
    3, 7, 6, 3, 6, 2,
    5, 1, 0, 5, 0, 4], dtype=np.int32).reshape(-1, 3)
CUBE_COLORS_RGBA8 = np.array([
    [255, 64, 64, 255], [64, 255, 64, 255], [64, 64, 255, 255], [255, 255, 64, 255],
    [255, 64, 255, 255], [64, 255, 255, 255], [200, 200, 200, 255], [32, 32, 32, 255]], dtype=np.float64)


def perspective(fov_deg: float, aspect: float, near: float, far: float) -> np.ndarray:
    """OpenGL-style projection; same rows as framework/base/Math.cpp:75-88 with x scaled by 1/aspect."""
    f = 1.0 / math.tan(math.radians(fov_deg) / 2.0)
    d = 1.0 / (near - far)
    return np.array([[f / aspect, 0, 0, 0], [0, f, 0, 0], [0, 0, (near + far) * d, 2 * near * far * d],
                     [0, 0, -1, 0]], dtype=np.float64)


def look_at(eye, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    eye, target, up = (np.asarray(v, dtype=np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def _records(clip: np.ndarray, rgba: np.ndarray) -> np.ndarray:
    v = np.empty((clip.shape[0], 8), dtype=np.float32)
    v[:, :4] = clip.astype(np.float32)
    v[:, 4:] = rgba.astype(np.float32)
    return v


def cube(width: int = 1024, height: int = 768, distance: float = 3.0) -> dict:
    """Config 1: the demo cube, fov 60, near 0.1, far 100, eye at `distance` from the origin."""
    eye = np.array([1.0, 1.2, 1.6])
    eye = eye / np.linalg.norm(eye) * distance
    mvp = perspective(60.0, width / height, 0.1, 100.0) @ look_at(eye, (0, 0, 0))
    pos = np.concatenate([CUBE_POSITIONS, np.ones((8, 1))], axis=1)
    clip = pos @ mvp.T
    rgba = (CUBE_COLORS_RGBA8.astype(np.float32) / np.float32(255.0)).astype(np.float32)
    return {"name": "cube", "vertices": _records(clip, rgba), "indices": CUBE_INDICES.copy(),
            "width": width, "height": height, "samples": 1}


def soup(num_tris: int, width: int, height: int, seed: int = 0, median_px: float = 4.0, sigma: float = 1.0,
         backface_frac: float = 0.5, alpha_range: tuple[float, float] | None = None, samples: int = 1) -> dict:
    """Config 2: non-indexed random soup. Centroids uniform over the clip-space box
    (NDC x, y in [-1, 1], z in [-1, 1]), w in [1, 10], lognormal screen-space edge
    length, random orientation, `backface_frac` reversed winding, RGBA8 colours."""
    rng = np.random.default_rng(seed)
    n = num_tris
    w = rng.uniform(1.0, 10.0, n)
    cx = rng.uniform(-1.0, 1.0, n)
    cy = rng.uniform(-1.0, 1.0, n)
    cz = rng.uniform(-1.0, 1.0, n)
    edge = np.exp(rng.normal(math.log(median_px), sigma, n))
    theta = rng.uniform(0.0, 2.0 * math.pi, n)
    r = edge / math.sqrt(3.0)
    k = np.arange(3)[None, :]
    jitter = rng.uniform(-0.35, 0.35, (n, 3))
    ang = theta[:, None] + (2.0 * math.pi / 3.0) * k + jitter
    px = r[:, None] * np.cos(ang)
    py = r[:, None] * np.sin(ang)
    back = rng.uniform(0.0, 1.0, n) < backface_frac
    px[back] = px[back][:, ::-1]
    py[back] = py[back][:, ::-1]
    nx = cx[:, None] + px * (2.0 / width)
    ny = cy[:, None] + py * (2.0 / height)
    nz = np.repeat(cz[:, None], 3, axis=1) + rng.uniform(-0.01, 0.01, (n, 3))
    nz = np.clip(nz, -1.0, 1.0)
    ww = np.repeat(w[:, None], 3, axis=1)
    clip = np.stack([nx * ww, ny * ww, nz * ww, ww], axis=-1).reshape(-1, 4)
    rgba = rng.integers(0, 256, (3 * n, 4)).astype(np.float32) / np.float32(255.0)
    if alpha_range is not None:
        a = rng.uniform(alpha_range[0], alpha_range[1], n)
        rgba[:, 3] = np.repeat((np.round(a * 255.0) / 255.0).astype(np.float32), 3)
    idx = np.arange(3 * n, dtype=np.int32).reshape(-1, 3)
    return {"name": f"soup{n}", "vertices": _records(clip, rgba.astype(np.float32)), "indices": idx,
            "width": width, "height": height, "samples": samples}


def value_noise(nx: int, ny: int, octaves: int = 6, seed: int = 0) -> np.ndarray:
    """Sum of `octaves` bilinear value-noise layers on an nx x ny grid, in [-1, 1]."""
    rng = np.random.default_rng(seed)
    out = np.zeros((ny, nx), dtype=np.float64)
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = 4 << o
        lattice = rng.uniform(-1.0, 1.0, (cells + 2, cells + 2))
        gx = np.linspace(0.0, cells, nx, endpoint=False)
        gy = np.linspace(0.0, cells, ny, endpoint=False)
        ix, iy = gx.astype(np.int64), gy.astype(np.int64)
        fx, fy = gx - ix, gy - iy
        fx = fx * fx * (3 - 2 * fx)
        fy = fy * fy * (3 - 2 * fy)
        a = lattice[np.ix_(iy, ix)]
        b = lattice[np.ix_(iy, ix + 1)]
        c = lattice[np.ix_(iy + 1, ix)]
        d = lattice[np.ix_(iy + 1, ix + 1)]
        top = a + (b - a) * fx[None, :]
        bot = c + (d - c) * fx[None, :]
        out += amp * (top + (bot - top) * fy[:, None])
        total += amp
        amp *= 0.5
    return out / total


def grid_mesh(n: int, seed: int = 0, amplitude: float = 0.2):
    """n x n vertex heightfield over [-1, 1]^2 (extent 2), heights = amplitude * extent * noise.
    Returns model-space positions [n*n, 3], colours [n*n, 4] and indices [2(n-1)^2, 3]."""
    h = value_noise(n, n, 6, seed) * amplitude * 2.0
    xs = np.linspace(-1.0, 1.0, n)
    X, Z = np.meshgrid(xs, xs)
    pos = np.stack([X, h, Z], axis=-1).reshape(-1, 3)
    t = (h.reshape(-1) / (amplitude * 2.0) + 1.0) * 0.5
    rgba = np.stack([0.2 + 0.6 * t, 0.5 + 0.3 * (1 - t), 0.25 + 0.2 * t, np.ones_like(t)], axis=-1)
    rgba = (np.round(rgba * 255.0) / 255.0).astype(np.float32)
    i = np.arange(n - 1)
    I, J = np.meshgrid(i, i)
    v00 = (J * n + I).reshape(-1)
    v10 = v00 + 1
    v01 = v00 + n
    v11 = v01 + 1
    tris = np.empty((2 * v00.size, 3), dtype=np.int32)
    tris[0::2] = np.stack([v00, v01, v10], axis=-1)
    tris[1::2] = np.stack([v10, v01, v11], axis=-1)
    return pos, rgba, tris


def terrain_eye_target(frame: float = 0.0, elevation_deg: float = 15.0):
    """Eye and target of the fly-through camera: a closed loop of 300 frames
    around the heightfield, looking across it at a grazing angle."""
    t = frame * 2.0 * math.pi / 300.0
    ex = 1.25 * math.sin(t)
    ez = 1.25 * math.cos(t)
    dist = math.hypot(ex, ez)
    ey = 0.25 + dist * math.tan(math.radians(elevation_deg)) * 0.5
    target = (0.3 * math.sin(t + 0.7), 0.0, 0.3 * math.cos(t + 0.7))
    return np.array([ex, ey, ez]), np.array(target)


def terrain_camera(frame: float = 0.0, width: int = 3840, height: int = 2160, elevation_deg: float = 15.0):
    """Camera at a grazing angle above the heightfield; `frame` moves it along a closed spline."""
    eye, target = terrain_eye_target(frame, elevation_deg)
    return perspective(60.0, width / height, 0.05, 10.0) @ look_at(eye, target)


def camera_delta(frame_a: float, frame_b: float, scale: float = 40.0) -> np.ndarray:
    """6 floats describing the camera move from frame_a to frame_b: the eye's
    displacement and the change of the unit view direction, both x scale."""
    ea, ta = terrain_eye_target(frame_a)
    eb, tb = terrain_eye_target(frame_b)
    fa = (ta - ea) / np.linalg.norm(ta - ea)
    fb = (tb - eb) / np.linalg.norm(tb - eb)
    return (np.concatenate([eb - ea, fb - fa]) * scale).astype(np.float32)


def water_mesh(n: int, level: float = -0.02, alpha: float = 0.35):
    """Flat translucent n x n grid over [-1, 1]^2 at height `level` (the
    fly-through's alpha-blended overlay layer)."""
    xs = np.linspace(-1.0, 1.0, n)
    X, Z = np.meshgrid(xs, xs)
    pos = np.stack([X, np.full_like(X, level), Z], axis=-1).reshape(-1, 3)
    ripple = 0.5 + 0.5 * np.sin(X * 37.0) * np.cos(Z * 29.0)
    rgba = np.stack([0.1 + 0.1 * ripple, 0.3 + 0.2 * ripple, 0.6 + 0.2 * ripple, np.full_like(X, alpha)], axis=-1)
    rgba = (np.round(rgba.reshape(-1, 4) * 255.0) / 255.0).astype(np.float32)
    i = np.arange(n - 1)
    I, J = np.meshgrid(i, i)
    v00 = (J * n + I).reshape(-1)
    tris = np.empty((2 * v00.size, 3), dtype=np.int32)
    tris[0::2] = np.stack([v00, v00 + n, v00 + 1], axis=-1)
    tris[1::2] = np.stack([v00 + 1, v00 + n, v00 + n + 1], axis=-1)
    return pos, rgba, tris


def terrain(n: int, width: int, height: int, samples: int = 1, seed: int = 0, frame: float = 0.0) -> dict:
    """Config 3 (n = 2048, 3840x2160, 4x MSAA) and the config 5 grid (n = 4096)."""
    pos, rgba, tris = grid_mesh(n, seed)
    mvp = terrain_camera(frame, width, height)
    clip = np.concatenate([pos, np.ones((pos.shape[0], 1))], axis=1) @ mvp.T
    return {"name": f"terrain{n}", "vertices": _records(clip, rgba), "indices": tris,
            "width": width, "height": height, "samples": samples, "mvp": mvp, "model": pos, "rgba": rgba}


def _mip_chain(img: np.ndarray) -> list[np.ndarray]:
    """Box-filtered mip levels of a square RGBA8 image [n, n, 4] (n a power of two)."""
    levels = [img]
    while levels[-1].shape[0] > 1:
        a = levels[-1].astype(np.uint32)
        b = (a[0::2, 0::2] + a[1::2, 0::2] + a[0::2, 1::2] + a[1::2, 1::2] + 2) // 4
        levels.append(b.astype(np.uint8))
    return levels


def texture_atlas(textures: list[np.ndarray], atlas_w: int = 256, atlas_h: int = 256):
    """Packs square RGBA8 textures and their mip chains into one atlas. Each texture
    takes a 2n x n strip holding its levels side by side from the left, top-aligned.
    Returns (atlas [H, W] uint32 with R in the low byte, [(size, mip_levels[L, 4])]) with
    mip_levels in the Material layout (scaleX, scaleY, biasX, biasY, normalized to the
    atlas)."""
    atlas = np.zeros((atlas_h, atlas_w, 4), np.uint8)
    specs, x0, y0, row_h = [], 0, 0, 0
    for tex in textures:
        n = tex.shape[0]
        if x0 + 2 * n > atlas_w:
            x0, y0 = 0, y0 + row_h
            row_h = 0
        assert y0 + n <= atlas_h, "atlas too small"
        levels, x = [], x0
        for k, lv in enumerate(_mip_chain(tex)):
            m = lv.shape[0]
            atlas[y0:y0 + m, x:x + m] = lv
            levels.append((m / atlas_w, m / atlas_h, x / atlas_w, y0 / atlas_h))
            x += m
        specs.append(((float(n), float(n)), np.array(levels, np.float32)))
        x0 += 2 * n
        row_h = max(row_h, n)
    words = atlas.astype(np.uint32)
    packed = words[..., 0] | (words[..., 1] << 8) | (words[..., 2] << 16) | (words[..., 3] << 24)
    return packed.astype(np.uint32), specs


def textured_terrain(n: int = 128, width: int = 640, height: int = 480, seed: int = 0, frame: float = 0.0,
                     tiles: float = 6.0) -> dict:
    """The heightfield as InputVertex records (position, normal, texture coordinate) for the
    textured Phong pipe, with four materials -- untextured; diffuse-textured; diffuse and
    alpha textured (the alpha test cuts holes); a second diffuse texture -- assigned per
    triangle, an atlas holding their mip chains, and the camera matrices."""
    rng = np.random.default_rng(seed)
    pos, _, tris = grid_mesh(n, seed)
    hgt = pos[:, 1].reshape(n, n)
    step = 2.0 / (n - 1)
    gx = np.gradient(hgt, step, axis=1)
    gz = np.gradient(hgt, step, axis=0)
    nrm = np.stack([-gx, np.ones_like(gx), -gz], axis=-1).reshape(-1, 3)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    uv = np.stack([(pos[:, 0] + 1.0) * 0.5 * tiles - tiles * 0.5, (pos[:, 2] + 1.0) * 0.5 * tiles], axis=-1)
    inp = np.concatenate([pos, nrm, uv], axis=1).astype(np.float32)

    def noise_tex(k, lo, hi):
        t = np.stack([value_noise(64, 64, 4, seed + k + c) for c in range(4)], axis=-1)
        t = (t - t.min()) / max(float(t.max() - t.min()), 1e-6)
        return np.clip(lo + (hi - lo) * t + rng.uniform(-0.08, 0.08, t.shape), 0, 1)

    texs = [(noise_tex(10, 0.1, 0.9) * 255).round().astype(np.uint8),
            (noise_tex(20, 0.0, 1.0) * 255).round().astype(np.uint8),
            (noise_tex(30, 0.2, 0.8) * 255).round().astype(np.uint8)]
    atlas, specs = texture_atlas(texs, 256, 128)
    from .raster import material_records
    materials = material_records(
        diffuse=[[0.7, 0.6, 0.5, 1.0], [1.0, 1.0, 1.0, 1.0], [1.0, 1.0, 1.0, 1.0], [1.0, 1.0, 1.0, 0.8]],
        specular=[[0.3, 0.3, 0.3], [0.5, 0.5, 0.4], [0.2, 0.2, 0.2], [0.8, 0.8, 0.8]],
        glossiness=[8.0, 32.0, 4.0, 96.0],
        diffuse_texture=[None, specs[0], specs[2], specs[2]],
        alpha_texture=[None, None, specs[1], None])
    tri_mat = rng.integers(0, 4, tris.shape[0]).astype(np.int32)
    eye, target = terrain_eye_target(frame, 25.0)
    view = look_at(eye, target).astype(np.float32)
    proj = perspective(60.0, width / height, 0.05, 10.0).astype(np.float32)
    return {"name": f"textured{n}", "input": inp, "indices": tris, "width": width, "height": height,
            "pos_to_clip": (proj @ view).astype(np.float32), "pos_to_camera": view,
            "normal_to_camera": view[:3, :3].copy(), "materials": materials, "triangle_material_idx": tri_mat,
            "atlas": atlas}


BATCH_RESOLUTIONS = [(256, 256), (512, 512), (1024, 768), (1920, 1080)]


def batch(count: int = 64, lo: int = 1000, hi: int = 500_000, seed: int = 0, blend_frac: float = 0.5) -> list[dict]:
    """Config 4: `count` soups, triangle counts log-uniform in [lo, hi], resolutions
    from BATCH_RESOLUTIONS, `blend_frac` of them alpha-blended (alpha in [0.2, 1])."""
    rng = np.random.default_rng(seed)
    scenes = []
    for i in range(count):
        n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        w, h = BATCH_RESOLUTIONS[int(rng.integers(0, len(BATCH_RESOLUTIONS)))]
        blended = i < int(round(count * blend_frac))
        s = soup(n, w, h, seed=seed * 1000 + i + 1, alpha_range=(0.2, 1.0) if blended else None)
        s["blend"] = "srcover" if blended else "replace"
        scenes.append(s)
    order = rng.permutation(count)
    return [scenes[i] for i in order]
