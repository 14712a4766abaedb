"""Autotuner for the run-time pipeline parameters (bin size, coarse unit size,
bin chunk size, fine warps per CTA) -- the reference's compile-time CR_*
constants (Constants.hpp:24-46) made tunable. Output bits never depend on
them (tests/test_gpu_batch.py::test_tuning_does_not_change_bits), so the
tuner only measures time.

    python cudaraster-linux_gb300/autotune.py [--workloads soup1m,batch64,subpixel,flythrough] [--out FILE]

Workloads: soup1m (1M-triangle soup at 1920x1080), batch64 (the uneven
64-scene batch replayed as one graph), subpixel (the grazing 2048^2
heightfield at 3840x2160, 4x MSAA) and flythrough (plain frames of the 4096^2
heightfield plus its water layer at 3840x2160, vertex transform fused into
setup). Writes {workload: {"best": {...}, "ms": best_ms, "candidates": [...]}}
to tuning.json next to this file; bench.py applies the entry of its workload.

The tile stays 8x8 pixels (the reference's CR_TILE_LOG2, Constants.hpp:41-46):
the fine stage's coverage masks, visibility keys and per-lane pixel ownership
are laid out for 64 pixels a tile, so tile size is not a run-time parameter.
"""
from __future__ import annotations

import argparse
import importlib
import itertools
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
PKG = HERE.name


SELF_PIXELS = (4, 8, 12, 16, 24, 32, 48, 64)


def candidates(quick: bool = False, medium: bool = False):
    bins = (3, 4, 5)
    warps = (4, 8)
    units = (0,) if quick else ((0, 64, 256) if medium else (0, 64, 128, 256, 512, 1024))
    chunks = (0,) if quick or medium else (0, 256, 1024, 4096)
    for b, w, u, c in itertools.product(bins, warps, units, chunks):
        yield {"bin_log2": b, "fine_warps": w, "coarse_unit_entries": u, "bin_chunk_tris": c}


def tune_single(scene: dict, pipe: str, cands, steps: int = 6, samples: int = 1) -> dict:
    import torch
    p = importlib.import_module(PKG)
    wl = importlib.import_module(PKG + ".workloads")
    W, H = scene["width"], scene["height"]
    color = p.CudaSurface((W, H), p.CudaSurface.FORMAT_RGBA8, samples)
    depth = p.CudaSurface((W, H), p.CudaSurface.FORMAT_DEPTH32, samples)
    v = torch.from_numpy(scene["vertices"]).cuda()
    i = torch.from_numpy(scene["indices"]).cuda()
    stream = torch.cuda.current_stream()
    results = []
    for t in cands:
        cr = p.CudaRaster()
        cr.init()
        try:
            cr.setTuning(**t)
        except p.RasterError:
            continue
        cr.setSurfaces(color, depth)
        cr.setPixelPipe(None, pipe)
        cr.setVertexBuffer(v, 0)
        cr.setIndexBuffer(i, 0, i.shape[0])

        def draw():
            cr.deferredClear(wl.CLEAR[:4], wl.CLEAR[4])
            cr.drawTriangles(stream)

        try:
            for _ in range(3):
                draw()
        except p.RasterError:   # e.g. more bins than one draw supports at this bin size
            continue
        ms = wl.time_events(draw, steps, stream)
        results.append({"tuning": t, "ms": sorted(ms)[len(ms) // 2]})
    results.sort(key=lambda r: r["ms"])
    return {"best": results[0]["tuning"], "ms": results[0]["ms"], "candidates": results}


def tune_flythrough(ft, cands, frames=(60, 140, 220), steps: int = 2) -> dict:
    """Median time of plain frames (terrain, then water) at a few camera
    positions of the loop, per candidate."""
    wl = importlib.import_module(PKG + ".workloads")
    p = importlib.import_module(PKG)
    import torch
    stream = torch.cuda.current_stream()
    results = []
    for t in cands:
        try:
            crs = ft.contexts(t)
        except p.RasterError:
            continue
        ms = []
        try:
            for f in frames:
                ft.frame_plain(crs, f, stream)   # warm: sizes this context's queues for the frame
                ms += wl.time_events(lambda: ft.frame_plain(crs, f, stream), steps, stream)
        except p.RasterError:
            continue
        finally:
            del crs
        results.append({"tuning": t, "ms": sorted(ms)[len(ms) // 2]})
    results.sort(key=lambda r: r["ms"])
    return {"best": results[0]["tuning"], "ms": results[0]["ms"], "candidates": results}


def tune_batch(batch, cands, steps: int = 4) -> dict:
    wl = importlib.import_module(PKG + ".workloads")
    p = importlib.import_module(PKG)
    import torch
    stream = torch.cuda.current_stream()
    results = []
    for t in cands:
        cr = p.CudaRaster()
        cr.init()
        try:
            cr.setTuning(**t)
        except p.RasterError:
            continue
        g = cr.createBatchGraph(batch.items)
        for _ in range(2):
            g.launch(stream)
        ms = wl.time_events(lambda: g.launch(stream), steps, stream)
        g.destroy()
        results.append({"tuning": t, "ms": sorted(ms)[len(ms) // 2]})
    results.sort(key=lambda r: r["ms"])
    return {"best": results[0]["tuning"], "ms": results[0]["ms"], "candidates": results}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workloads", default="soup1m,batch64")
    ap.add_argument("--out", default=str(HERE / "tuning.json"))
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--grid", choices=["full", "medium"], default="full",
                    help="medium: bins x warps x three unit sizes, for the large workloads")
    args = ap.parse_args()
    scenes = importlib.import_module(PKG + ".scenes")
    wl = importlib.import_module(PKG + ".workloads")
    out = json.loads(Path(args.out).read_text()) if Path(args.out).exists() else {}
    cands = list(candidates(args.quick, args.grid == "medium"))
    for name in args.workloads.split(","):
        if name == "soup1m":
            scene = scenes.soup(1_000_000, 1920, 1080, seed=2)
            run = lambda c: tune_single(scene, "PixelPipe_gouraud", c)  # noqa: E731
        elif name == "batch64":
            batch = wl.Batch(scenes.batch(64, seed=4))
            run = lambda c: tune_batch(batch, c)  # noqa: E731
        elif name == "subpixel":
            scene = scenes.terrain(2048, 3840, 2160, 4, seed=5, frame=120.0)
            run = lambda c: tune_single(scene, "PixelPipe_gouraud_msaa4", c, samples=4)  # noqa: E731
        elif name == "flythrough":
            ft = wl.FlyThrough()
            run = lambda c: tune_flythrough(ft, c)  # noqa: E731
        else:
            raise SystemExit(f"unknown workload {name}")
        res = run(cands)
        if not args.quick:
            # Second pass: the fine stage's self-rasterization threshold around the best grid point.
            extra = run([dict(res["best"], fine_self_pixels=v) for v in SELF_PIXELS])
            allc = sorted(res["candidates"] + extra["candidates"], key=lambda r: r["ms"])
            res = {"best": allc[0]["tuning"], "ms": allc[0]["ms"], "candidates": allc}
        out[name] = res
        print(name, out[name]["best"], out[name]["ms"], flush=True)
        Path(args.out).write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
