"""Per-stage check of the bin and coarse stages: the GPU's bin and tile lists,
read back with cr_read_queue_output, against the oracle's queue model.

For every bin and every 8x8 tile the GPU list must be
  (a) a superset of the exact list (entries covering a sample of the cell),
  (b) strictly increasing, i.e. in submission order (triangle, subtriangle),
  (c) free of entries whose bounding box misses the cell,
and equal to the list of the documented conservative rule (bounding box, then
the edge-versus-rectangle test for boxes larger than 2x2 cells). The
reference emits its lists in the same order (BinRaster.inl:381-418,
CoarseRaster.inl:561-680) from conservative tests of the same kind
(BinRaster.inl:228-300)."""
import ctypes as C

import numpy as np
import pytest

from conftest import pkg_mod
from helpers import PIPES, PIPE_SAMPLES, gpu_render, pkg, vertices_for
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _near_clipped_soup():
    sc = pkg_mod("scenes").soup(4000, 256, 200, seed=9, median_px=400.0, sigma=1.2)
    v = sc["vertices"].copy()
    v[::7, 2] = -1.5 * v[::7, 3]   # through the near plane: clipped into several subtriangles
    sc["vertices"] = v
    return sc


SCENES = {
    "soup": lambda: pkg_mod("scenes").soup(20000, 320, 240, seed=31, median_px=6.0),
    "large": lambda: pkg_mod("scenes").soup(3000, 640, 360, seed=32, median_px=60.0, sigma=1.0),
    "near_clipped": _near_clipped_soup,
    "odd_viewport": lambda: pkg_mod("scenes").soup(8000, 331, 197, seed=33, median_px=12.0),
}


def _gpu_queues(cr, lib):
    nb, nt = C.c_int64(), C.c_int64()
    assert lib.cr_read_queue_output(cr._ctx, None, None, None, 0, None, None, None, 0, C.byref(nb), C.byref(nt)) == 0
    cnt = cr.getCounters()
    bs, bc = np.zeros(cnt["num_bins"], np.int32), np.zeros(cnt["num_bins"], np.int32)
    ts, tc = np.zeros(cnt["num_tiles"], np.int32), np.zeros(cnt["num_tiles"], np.int32)
    bl, tl = np.zeros(max(nb.value, 1), np.uint32), np.zeros(max(nt.value, 1), np.uint32)
    st = lib.cr_read_queue_output(cr._ctx, bs.ctypes.data, bc.ctypes.data, bl.ctypes.data, bl.shape[0],
                                  ts.ctypes.data, tc.ctypes.data, tl.ctypes.data, tl.shape[0], C.byref(nb),
                                  C.byref(nt))
    assert st == 0
    return (bs, bc, bl), (ts, tc, tl)


def _check_level(level, gpu, exact, rule, what):
    starts, counts, flat = gpu
    eo, ee = exact
    ro, re_ = rule
    assert len(starts) == len(eo) - 1, f"{what}: {len(starts)} {level}s, oracle {len(eo) - 1}"
    n_exact = n_gpu = 0
    for c in range(len(starts)):
        g = flat[starts[c]:starts[c] + counts[c]].astype(np.int64)
        e = ee[eo[c]:eo[c + 1]].astype(np.int64)
        r = re_[ro[c]:ro[c + 1]].astype(np.int64)
        assert np.all(np.diff(g) > 0), f"{what}: {level} {c} not in submission order"
        missing = np.setdiff1d(e, g)
        assert missing.size == 0, f"{what}: {level} {c} lacks covering entries {missing[:8]}"
        assert np.array_equal(g, r), (f"{what}: {level} {c}: gpu {g.size} entries, rule {r.size}; extra "
                                      f"{np.setdiff1d(g, r)[:8]}, missing {np.setdiff1d(r, g)[:8]}")
        n_exact += e.size
        n_gpu += g.size
    return n_exact, n_gpu


def _bbox_misses(flat, starts, counts, hdr, width, height, cell_log2, per_row):
    """How many entries of the cells' lists have a bounding box (from the oracle's setup
    headers) that misses their cell."""
    cell = np.repeat(np.arange(len(starts)), counts)
    idx = np.concatenate([np.arange(s, s + c) for s, c in zip(starts, counts)] or [np.zeros(0, np.int64)])
    e = flat[idx].astype(np.int64)
    t, k = e >> 3, e & 7
    slot = np.where(k == 7, t, hdr[t, 3].astype(np.int64) + k)
    w = hdr[slot, :3].astype(np.int64)
    xs = (w & 0xFFFF).astype(np.int16).astype(np.int64) + (width << 3)
    ys = (w >> 16).astype(np.int16).astype(np.int64) + (height << 3)
    cx, cy = cell % per_row, cell // per_row
    inside = ((xs.min(1) >> cell_log2) <= cx) & (cx <= (xs.max(1) >> cell_log2)) & \
             ((ys.min(1) >> cell_log2) <= cy) & (cy <= (ys.max(1) >> cell_log2))
    return int((~inside).sum())


@pytest.mark.parametrize("pipe", ["PixelPipe_gouraud", "PixelPipe_gouraud_msaa4"])
@pytest.mark.parametrize("scene", list(SCENES))
@pytest.mark.parametrize("bin_log2", [3, 4, 5])
def test_queues_match_oracle_model(cuda, pipe, scene, bin_log2):
    p = pkg()
    lib = pkg_mod("_lib").load()
    sc = SCENES[scene]()
    cr = p.CudaRaster()
    cr.init()
    cr.setTuning(bin_log2=bin_log2)
    clear = (p.color_to_abgr(0.1, 0.2, 0.3, 1.0), p.clear_depth_from_float(1.0))
    gpu_render(pipe, sc, clear, cr=cr)
    bins, tiles = _gpu_queues(cr, lib)
    flags, blend, shader, stride = PIPES[pipe]
    op = orc.make_pipe(sc["width"], sc["height"], PIPE_SAMPLES.get(pipe, 1), flags, blend, shader, stride)
    v = vertices_for(pipe, sc["vertices"])
    q = {k: orc.queue_lists(op, v, sc["indices"], bin_log2, k) for k in orc.QUEUE_KINDS}
    what = f"{pipe} {scene} bins of {8 << bin_log2} px"
    eb, gb = _check_level("bin", bins, q["bin_exact"], q["bin_rule"], what)
    et, gt = _check_level("tile", tiles, q["tile_exact"], q["tile_rule"], what)
    assert eb > 0 and et > 0
    # Conservative but not wasteful: the rule keeps few entries beyond the exact ones.
    assert gt <= 1.6 * et + 64, f"{what}: {gt} tile entries for {et} covering ones"


def test_queue_entries_touch_their_cells(cuda):
    """(c) checked directly from the setup headers, independently of the rule's model."""
    p = pkg()
    lib = pkg_mod("_lib").load()
    sc = _near_clipped_soup()
    cr = p.CudaRaster()
    cr.init()
    gpu_render("PixelPipe_gouraud", sc, None, cr=cr)
    (bs, bc, bl), (ts, tc, tl) = _gpu_queues(cr, lib)
    op = orc.make_pipe(sc["width"], sc["height"], 1, orc.DEPTH | orc.LERP, "replace", "gouraud", 32)
    _, hdr, _, _ = orc.setup(op, sc["vertices"], sc["indices"])
    w, h = sc["width"], sc["height"]
    wt = (w + 7) >> 3
    wb = (wt + 15) >> 4
    assert _bbox_misses(bl, bs, bc, hdr, w, h, 4 + 3 + 4, wb) == 0
    assert _bbox_misses(tl, ts, tc, hdr, w, h, 4 + 3, wt) == 0
    assert int(tc.sum()) == tl.shape[0] and int(bc.sum()) == bl.shape[0]


def test_read_queue_output_validation(cuda):
    p = pkg()
    lib = pkg_mod("_lib").load()
    cr = p.CudaRaster()
    cr.init()
    nb, nt = C.c_int64(), C.c_int64()
    # No draw yet: not a single draw.
    assert lib.cr_read_queue_output(cr._ctx, None, None, None, 0, None, None, None, 0, C.byref(nb), C.byref(nt)) == 2
    sc = pkg_mod("scenes").soup(2000, 128, 96, seed=34)
    gpu_render("PixelPipe_gouraud", sc, None, cr=cr)
    assert lib.cr_read_queue_output(cr._ctx, None, None, None, 0, None, None, None, 0, C.byref(nb), C.byref(nt)) == 0
    assert nb.value > 0 and nt.value > 0
    small = np.zeros(1, np.uint32)
    assert lib.cr_read_queue_output(cr._ctx, None, None, small.ctypes.data, 1, None, None, None, 0, C.byref(nb),
                                    C.byref(nt)) == 5
