"""Benchmark workloads shared by bench.py and the autotuner.

uneven batch (64 soups of 1k..500k triangles, mixed resolutions, half of them
alpha-blended): the plain path draws the scenes one after another with
drawTriangles (each draw reads its counters back, as the reference does); the
batched path replays one captured CUDA graph that draws all of them. Both are
timed with CUDA events on the drawing stream and checked bit for bit against
each other.
"""
from __future__ import annotations

import importlib
import json
from pathlib import Path

import numpy as np
import torch

PKG = __name__.rsplit(".", 1)[0]
TUNING_FILE = Path(__file__).resolve().parent / "tuning.json"
CLEAR = (0.1, 0.2, 0.3, 1.0, 1.0)


def _pkg():
    return importlib.import_module(PKG)


def load_tuning(workload: str) -> dict:
    if TUNING_FILE.exists():
        return json.loads(TUNING_FILE.read_text()).get(workload, {}).get("best", {})
    return {}


class Batch:
    """Scenes of a batch resident on the GPU with their surfaces."""

    def __init__(self, scenes: list[dict]):
        p = _pkg()
        self.items = []
        for sc in scenes:
            pipe = "PixelPipe_gouraud_srcover" if sc.get("blend") == "srcover" else "PixelPipe_gouraud"
            cs = p.CudaSurface((sc["width"], sc["height"]), p.CudaSurface.FORMAT_RGBA8, 1)
            ds = p.CudaSurface((sc["width"], sc["height"]), p.CudaSurface.FORMAT_DEPTH32, 1)
            v = torch.from_numpy(sc["vertices"]).cuda()
            i = torch.from_numpy(np.ascontiguousarray(sc["indices"], dtype=np.int32)).cuda()
            self.items.append({"pipe": pipe, "color": cs, "depth": ds, "vertices": v, "indices": i,
                               "numTris": int(i.shape[0]), "clear": CLEAR})
        self.num_tris = sum(it["numTris"] for it in self.items)

    def snapshot(self):
        return [(it["color"].tensor.clone(), it["depth"].tensor.clone()) for it in self.items]


def draw_plain(cr, batch: Batch, stream) -> None:
    """The reference's usage: one scene at a time through drawTriangles."""
    for it in batch.items:
        cr.setSurfaces(it["color"], it["depth"])
        cr.setPixelPipe(None, it["pipe"])
        cr.deferredClear(CLEAR[:4], CLEAR[4])
        cr.setVertexBuffer(it["vertices"], 0)
        cr.setIndexBuffer(it["indices"], 0, it["numTris"])
        cr.drawTriangles(stream)


def time_events(fn, steps: int, stream) -> list[float]:
    out = []
    for _ in range(steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        out.append(a.elapsed_time(b))
    return out


def measure_batch(batch: Batch, steps: int = 5, warmup: int = 3, tuning: dict | None = None) -> dict:
    """Plain sequential draws vs one graph replay of the whole batch."""
    p = _pkg()
    stream = torch.cuda.current_stream()
    plain = p.CudaRaster()
    plain.init()
    for _ in range(warmup):
        draw_plain(plain, batch, stream)
    torch.cuda.synchronize()
    plain_ms = time_events(lambda: draw_plain(plain, batch, stream), steps, stream)
    ref = batch.snapshot()

    cr = p.CudaRaster()
    cr.init()
    if tuning:
        cr.setTuning(**tuning)
    graph = cr.createBatchGraph(batch.items)
    for _ in range(warmup):
        graph.launch(stream)
    torch.cuda.synchronize()
    batched_ms = time_events(lambda: graph.launch(stream), steps, stream)
    counters = graph.counters(stream)
    got = batch.snapshot()
    exact = all(torch.equal(a[0], b[0]) and torch.equal(a[1], b[1]) for a, b in zip(ref, got))
    graph.destroy()
    plain_t = sum(plain_ms) / len(plain_ms)
    batch_t = sum(batched_ms) / len(batched_ms)
    return {"scenes": len(batch.items), "num_tris": batch.num_tris,
            "plain_ms_per_batch": round(plain_t, 4), "batched_ms_per_batch": round(batch_t, 4),
            "plain_frames_per_s": round(1000.0 / plain_t, 3), "batched_frames_per_s": round(1000.0 / batch_t, 3),
            "speedup": round(plain_t / batch_t, 3), "batched_mtri_per_s": round(batch.num_tris / batch_t / 1e3, 2),
            "bit_exact_vs_plain": bool(exact), "overflow": counters["overflow"], "tuning": tuning or {}}
