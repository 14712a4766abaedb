"""The fly-through with the learned queue predictor, at reduced size (a 1024^2
heightfield and its water layer at 1920x1080): over 60 frames (the first 20
plain) every frame of the pipelined, predictor-sized path is bit-identical to
the plain path, a frame matches the CPU oracle, and forced misses are caught
by the overflow flags and redrawn exactly; over the whole 300-frame loop (the
first 50 plain) the predictor sizes the queues more tightly than the
previous-frame sizing of the reference. Whether the trained network also beats
the trend extrapolation it starts from is recorded by an expected failure."""
import math

import numpy as np
import pytest
import torch

from conftest import pkg_mod
from helpers import assert_same, oracle_render, pkg
from oracle import vertex_oracle

pytestmark = pytest.mark.gpu

N, W, H, FRAMES, TRAIN = 1024, 1920, 1080, 60, 20
LOOP, LOOP_TRAIN = 300, 50


@pytest.fixture(scope="module")
def fly(cuda):
    return pkg_mod("workloads").FlyThrough(n=N, width=W, height=H, frames=LOOP, seed=5)


@pytest.fixture(scope="module")
def plain(fly):
    keep = (TRAIN, 30, FRAMES - 1)
    _, sums, kept, _ = pkg_mod("workloads").run_flythrough_plain(fly, range(FRAMES), checksums=True, keep=keep)
    return sums, kept, keep


def _same_frames(res, plain):
    sums, kept, keep = plain
    assert res["checksums"] == sums
    for f in keep:
        assert torch.equal(kept[f][0], res["kept"][f][0]) and torch.equal(kept[f][1], res["kept"][f][1]), f


def test_predicted_frames_are_bit_exact(fly, plain):
    res = pkg_mod("workloads").run_flythrough_predicted(fly, FRAMES, TRAIN, checksums=True, keep=plain[2])
    _same_frames(res, plain)
    assert len(res["records"]) == 2 * (FRAMES - TRAIN)
    assert all(r["bin"] > 0 and r["tile"] > 0 for r in res["records"])
    assert all(s > 0 for s in res["adam_steps"])


def test_forced_misses_are_redrawn_exactly(fly, plain):
    # Capacities at half the prediction: every predicted frame overflows and
    # the plain overflow-detect-and-rerun path redraws it.
    res = pkg_mod("workloads").run_flythrough_predicted(fly, FRAMES, TRAIN, checksums=True, keep=plain[2],
                                                        capacity_scale=0.5)
    assert res["misses"] == [FRAMES - TRAIN] * 2
    assert all(r["miss"] for r in res["records"])
    _same_frames(res, plain)


def test_flythrough_frame_matches_oracle(fly, plain):
    p = pkg()
    raster = pkg_mod("raster")
    wl = pkg_mod("workloads")
    f = 30
    gc = plain[1][f][0].cpu().numpy().view(np.uint32)
    gd = plain[1][f][1].cpu().numpy().view(np.uint32)
    mvp = fly.mvps[f]
    clear = (p.color_to_abgr(*wl.WATER_CLEAR[:4]), p.clear_depth_from_float(wl.WATER_CLEAR[4]))
    color = depth = None
    for k, (layer, pipe) in enumerate(zip(fly.layers, ("PixelPipe_gouraud", "PixelPipe_gouraud_srcover"))):
        clip = vertex_oracle.vertex_passthrough(layer["model"].cpu().numpy(), mvp)
        verts = np.concatenate([clip, layer["colors"].cpu().numpy()], axis=1).astype(np.float32)
        sc = {"vertices": verts, "indices": layer["indices"].cpu().numpy(), "width": W, "height": H}
        color, depth, st = oracle_render(pipe, sc, clear if k == 0 else None, color, depth)
        assert st["zmin_violations"] == 0
    assert_same(gc, gd, color, depth, f"fly-through frame {f}")


@pytest.fixture(scope="module")
def loop(fly):
    """The whole 300-frame loop, the first 50 frames plain, the rest predictor-sized."""
    return pkg_mod("workloads").run_flythrough_predicted(fly, LOOP, LOOP_TRAIN)


def _errors(loop):
    """Mean absolute log error of the bin / tile totals sized two frames ahead, per
    layer: the predictor, the reference's sizing from the last draw it has seen,
    and trend extrapolation alone (what the network predicts untrained)."""
    out = {}
    for k in range(2):
        r = sorted((x for x in loop["records"] if x["layer"] == k), key=lambda x: x["frame"])
        for q in ("bin", "tile"):
            a = np.array([x[q] for x in r], np.float64)
            p = np.array([x["pred_" + q] for x in r], np.float64)
            tgt = a[3:]
            out[(k, q)] = {"predictor": float(np.abs(np.log(tgt / p[3:])).mean()),
                           "previous_frame": float(np.abs(np.log(tgt / a[1:-2])).mean()),
                           "trend_only": float(np.abs(np.log(tgt / (a[1:-2] ** 3 / a[:-3] ** 2))).mean())}
    return out


def test_predictor_sizes_tighter_than_previous_frame_sizing(loop):
    assert loop["misses"] == [0, 0] or sum(loop["misses"]) <= 2
    for key, e in _errors(loop).items():
        assert math.isfinite(e["predictor"])
        assert e["predictor"] < e["previous_frame"], (key, e)


@pytest.mark.xfail(reason="on this camera loop the trend's residual of the queue totals is not predictable from the "
                          "network's inputs (pooled histogram, camera move): a least-squares fit on them removes "
                          "about 2% of it even in sample, and the trained correction ties or loses to the trend",
                   strict=False)
def test_trained_beats_trend_only(loop):
    errs = _errors(loop)
    print({f"{k}/{q}": {n: round(v, 5) for n, v in e.items()} for (k, q), e in errs.items()})
    for key, e in errs.items():
        assert e["predictor"] < e["trend_only"], (key, e)
