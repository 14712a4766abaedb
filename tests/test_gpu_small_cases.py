"""Small cases against the CPU oracle and against properties that need no
oracle: the fill rule on shared edges (every pixel of a closed mesh covered
exactly once), degenerate and edge-on triangles (nothing drawn), sweeps of 1
to 64 triangles of every size, and repeated draws giving the same bits."""
import numpy as np
import pytest

from helpers import assert_same, gpu_render, oracle_render, pkg

pytestmark = pytest.mark.gpu


def _records(px, py, w, h, rgba, z=0.0):
    """GouraudVertex records from pixel-space positions (y up, w = 1)."""
    n = px.size
    v = np.zeros((n, 8), np.float32)
    v[:, 0] = px / w * 2.0 - 1.0
    v[:, 1] = py / h * 2.0 - 1.0
    v[:, 2] = z
    v[:, 3] = 1.0
    v[:, 4:8] = rgba
    return v


def _grid_mesh(w, h, nx, ny, seed):
    """A closed mesh of nx x ny quads (two triangles each) over the whole viewport and
    beyond, its inner vertices jittered to sub-pixel positions, so edges are shared at
    every angle."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(-8.0, w + 8.0, nx + 1)
    ys = np.linspace(-8.0, h + 8.0, ny + 1)
    X, Y = np.meshgrid(xs, ys)
    # At most 0.2 of a cell: every quad stays convex, so its two triangles tile it.
    jx = rng.uniform(-0.2, 0.2, X.shape) * (w + 16) / nx
    jy = rng.uniform(-0.2, 0.2, Y.shape) * (h + 16) / ny
    jx[[0, -1], :] = 0
    jx[:, [0, -1]] = 0
    jy[[0, -1], :] = 0
    jy[:, [0, -1]] = 0
    px, py = (X + jx).reshape(-1), (Y + jy).reshape(-1)
    i = np.arange(nx)
    I, J = np.meshgrid(i, np.arange(ny))
    v00 = (J * (nx + 1) + I).reshape(-1)
    tris = np.empty((2 * v00.size, 3), np.int32)
    tris[0::2] = np.stack([v00, v00 + 1, v00 + nx + 1], -1)
    tris[1::2] = np.stack([v00 + 1, v00 + nx + 2, v00 + nx + 1], -1)
    # Alternate the winding of every other quad's diagonal: both diagonals occur.
    flip = (I + J).reshape(-1) % 2 == 1
    t0 = tris[0::2].copy()
    t1 = tris[1::2].copy()
    t0[flip] = np.stack([v00[flip], v00[flip] + 1, v00[flip] + nx + 2], -1)
    t1[flip] = np.stack([v00[flip], v00[flip] + nx + 2, v00[flip] + nx + 1], -1)
    tris[0::2], tris[1::2] = t0, t1
    return px, py, tris


def _fan(w, h, k, seed):
    rng = np.random.default_rng(seed)
    cx, cy = w / 2 + rng.uniform(-0.5, 0.5), h / 2 + rng.uniform(-0.5, 0.5)
    ang = np.sort(rng.uniform(0, 2 * np.pi, k))
    r = max(w, h) * 2.0
    px = np.concatenate([[cx], cx + r * np.cos(ang)])
    py = np.concatenate([[cy], cy + r * np.sin(ang)])
    tris = np.stack([np.zeros(k, np.int32), 1 + np.arange(k), 1 + (np.arange(k) + 1) % k], -1).astype(np.int32)
    return px, py, tris


@pytest.mark.parametrize("mesh", ["grid", "fan"])
@pytest.mark.parametrize("samples_pipe", [(1, "PixelPipe_gouraud_nodepth")])
def test_shared_edges_cover_every_pixel_once(cuda, mesh, samples_pipe):
    # Without depth test and with src-over at alpha 1/2, a pixel covered twice (or not
    # at all) differs from one blend of the colour over the clear colour.
    p = pkg()
    w, h = 97, 61
    if mesh == "grid":
        px, py, tris = _grid_mesh(w, h, 13, 9, seed=4)
    else:
        px, py, tris = _fan(w, h, 37, seed=5)
    # Channels a quarter step above a byte value: interpolation rounding cannot move them.
    rgba = (np.array([200.25, 100.25, 50.25, 128.25], np.float32) / 255.0).astype(np.float32)
    sc = {"vertices": _records(px, py, w, h, rgba), "indices": tris, "width": w, "height": h}
    clear = (p.color_to_abgr(0.0, 0.0, 0.0, 1.0), p.clear_depth_from_float(1.0))
    gc, gd, _, _ = gpu_render(samples_pipe[1], sc, clear)
    rc, rd, _ = oracle_render(samples_pipe[1], sc, clear)
    assert_same(gc, gd, rc, rd, f"{mesh} shared edges")
    img = gc[:h, :w]
    once = np.unique(img)
    assert once.size == 1 and once[0] != clear[0], f"{mesh}: pixel values {once[:8]}"


def test_degenerate_and_edge_on_triangles_draw_nothing(cuda):
    # Points on the 1/16-pixel snap grid of a 64 x 64 viewport (their NDC values and
    # snapped positions are exact): collinear triples and triangles with a repeated
    # vertex have zero area after snapping, so nothing is drawn.
    p = pkg()
    w = h = 64
    rng = np.random.default_rng(7)
    px, py, tris = [], [], []
    for k in range(40):
        a = rng.integers(0, 64 * 16, 2)
        d = rng.integers(-64, 65, 2) * 4
        j = int(rng.integers(0, 5))
        trip = [a, a + d, a + d * j // 4] if k < 30 else [a, a, a + d]
        for q in trip:
            px.append(q[0] / 16.0)
            py.append(q[1] / 16.0)
        tris.append([3 * k, 3 * k + 1, 3 * k + 2])
    sc = {"vertices": _records(np.array(px), np.array(py), w, h, np.array([1, 1, 1, 1], np.float32)),
          "indices": np.array(tris, np.int32), "width": w, "height": h}
    clear = (p.color_to_abgr(0.0, 0.0, 0.0, 1.0), p.clear_depth_from_float(1.0))
    gc, gd, _, _ = gpu_render("PixelPipe_gouraud", sc, clear)
    rc, rd, st = oracle_render("PixelPipe_gouraud", sc, clear)
    assert_same(gc, gd, rc, rd, "degenerate")
    assert st["num_fragments"] == 0
    assert (gc[:h, :w] == clear[0]).all()


@pytest.mark.parametrize("pipe", ["PixelPipe_gouraud", "PixelPipe_gouraud_msaa4", "PixelPipe_gouraud_srcover",
                                  "PixelPipe_gouraud_additive", "PixelPipe_trihash_srcover"])
@pytest.mark.parametrize("n", [1, 2, 3, 7, 31, 32, 33, 64])
def test_small_sweeps_match_oracle(cuda, pipe, n):
    p = pkg()
    scenes = __import__("conftest").pkg_mod("scenes")
    for k, median in enumerate((0.3, 2.0, 12.0, 80.0)):
        sc = scenes.soup(n, 72, 40, seed=1000 * n + k, median_px=median, sigma=1.0,
                         alpha_range=(0.2, 1.0) if "srcover" in pipe or "additive" in pipe else None)
        clear = (p.color_to_abgr(0.3, 0.2, 0.1, 1.0), p.clear_depth_from_float(1.0))
        gc, gd, _, _ = gpu_render(pipe, sc, clear)
        rc, rd, st = oracle_render(pipe, sc, clear)
        assert st["zmin_violations"] == 0
        assert_same(gc, gd, rc, rd, f"{pipe} n={n} median={median}")


@pytest.mark.parametrize("pipe", ["PixelPipe_gouraud", "PixelPipe_gouraud_srcover", "PixelPipe_gouraud_msaa4"])
def test_repeated_draws_are_identical(cuda, pipe):
    p = pkg()
    scenes = __import__("conftest").pkg_mod("scenes")
    sc = scenes.soup(30000, 320, 240, seed=77, median_px=8.0,
                     alpha_range=(0.2, 1.0) if "srcover" in pipe else None)
    clear = (p.color_to_abgr(0.3, 0.2, 0.1, 1.0), p.clear_depth_from_float(1.0))
    cr = p.CudaRaster()
    cr.init()
    first = gpu_render(pipe, sc, clear, cr=cr)
    for _ in range(4):
        again = gpu_render(pipe, sc, clear, cr=cr)
        assert_same(again[0], again[1], first[0], first[1], f"{pipe} repeat")


@pytest.mark.parametrize("pipe", ["PixelPipe_gouraud", "PixelPipe_gouraud_msaa4", "PixelPipe_gouraud_srcover"])
def test_equal_depth_copies_keep_the_first(cuda, pipe):
    """Every triangle drawn three times with the same positions (equal depths at
    every sample) and different colours, the copies scattered through the
    submission order: under depth LESS the first copy submitted keeps every
    sample -- through the visibility keys of the depth-resolved pipes, whose
    ties go to the lower list position, and through the ordered path."""
    from conftest import pkg_mod
    from helpers import PIPE_SAMPLES
    base = pkg_mod("scenes").soup(3000, 256, 192, seed=51, median_px=10.0,
                                  alpha_range=(0.2, 1.0) if "srcover" in pipe else None)
    rng = np.random.default_rng(52)
    T = base["indices"].shape[0]
    verts = []
    for _ in range(3):
        v = base["vertices"].copy()
        v[:, 4:8] = (np.round(rng.uniform(0, 1, (v.shape[0], 4)) * 255) / 255).astype(np.float32)
        verts.append(v)
    V = base["vertices"].shape[0]
    allv = np.concatenate(verts)
    tris = np.concatenate([base["indices"] + k * V for k in range(3)])
    order = rng.permutation(3 * T)
    sc = dict(base, vertices=allv, indices=np.ascontiguousarray(tris[order], dtype=np.int32))
    sc["samples"] = PIPE_SAMPLES.get(pipe, 1)
    p = pkg()
    clear = (p.color_to_abgr(0.1, 0.1, 0.1, 1.0), p.clear_depth_from_float(1.0))
    gc, gd, _, _ = gpu_render(pipe, sc, clear)
    rc, rd, st = oracle_render(pipe, sc, clear)
    assert st["zmin_violations"] == 0
    assert_same(gc, gd, rc, rd, f"{pipe} equal-depth copies")
