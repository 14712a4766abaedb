"""Autotuner for the run-time pipeline parameters (bin size, coarse unit size,
bin chunk size, fine warps per CTA) -- the reference's compile-time CR_*
constants (Constants.hpp:24-46) made tunable. Output bits never depend on
them (tests/test_gpu_batch.py::test_tuning_does_not_change_bits), so the
tuner only measures time.

    python cudaraster-linux_gb300/autotune.py [--workloads soup1m,batch64] [--out FILE]

Writes {workload: {"best": {...}, "ms": best_ms, "candidates": [...]}} to
tuning.json next to this file; bench.py applies the entry of its workload.
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


def candidates(quick: bool = False):
    bins = (3, 4, 5)
    warps = (4, 8)
    units = (0, 64, 128, 256, 512, 1024) if not quick else (0,)
    chunks = (0, 256, 1024, 4096) if not quick else (0,)
    for b, w, u, c in itertools.product(bins, warps, units, chunks):
        yield {"bin_log2": b, "fine_warps": w, "coarse_unit_entries": u, "bin_chunk_tris": c}


def tune_single(scene: dict, pipe: str, cands, steps: int = 6) -> dict:
    import torch
    p = importlib.import_module(PKG)
    wl = importlib.import_module(PKG + ".workloads")
    W, H = scene["width"], scene["height"]
    color = p.CudaSurface((W, H), p.CudaSurface.FORMAT_RGBA8, 1)
    depth = p.CudaSurface((W, H), p.CudaSurface.FORMAT_DEPTH32, 1)
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

        for _ in range(3):
            draw()
        ms = wl.time_events(draw, steps, stream)
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
    args = ap.parse_args()
    scenes = importlib.import_module(PKG + ".scenes")
    wl = importlib.import_module(PKG + ".workloads")
    out = json.loads(Path(args.out).read_text()) if Path(args.out).exists() else {}
    cands = list(candidates(args.quick))
    for name in args.workloads.split(","):
        if name == "soup1m":
            scene = scenes.soup(1_000_000, 1920, 1080, seed=2)
            run = lambda c: tune_single(scene, "PixelPipe_gouraud", c)  # noqa: E731
        elif name == "batch64":
            batch = wl.Batch(scenes.batch(64, seed=4))
            run = lambda c: tune_batch(batch, c)  # noqa: E731
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
