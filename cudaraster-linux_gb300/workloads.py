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


# ---------------------------------------------------------------- fly-through
WATER_CLEAR = (0.05, 0.1, 0.2, 1.0, 1.0)


class FlyThrough:
    """Camera fly-through over an n x n heightfield (2(n-1)^2 triangles) at
    width x height, depth LESS, followed every frame by a translucent water
    layer with about `overlay_frac` of the terrain's triangle count drawn
    src-over on the same surfaces. Each frame transforms the vertices -- fused
    into the setup stage (cr_set_vertex_transform: clip positions computed
    from the model positions and the frame's MVP, the colour varyings read
    from one static record buffer per layer), or with fused=False by the
    separate vertex stage (cr_vertex_shader_passthrough) into one of three
    record buffers -- then runs the opaque draw (with a deferred clear) and
    the overlay draw into one of two colour/depth surface pairs. Both give the
    same bits."""

    VERTEX_SLOTS = 3
    TARGETS = 2

    def __init__(self, n: int = 4096, width: int = 3840, height: int = 2160, frames: int = 300, seed: int = 5,
                 overlay_frac: float = 0.1, water_level: float = -0.02, water_alpha: float = 0.35,
                 fused: bool = True):
        import math
        p = _pkg()
        scenes = importlib.import_module(PKG + ".scenes")
        self.raster = importlib.import_module(PKG + ".raster")
        self.scenes = scenes
        self.n, self.width, self.height, self.frames = n, width, height, frames
        self.fused = fused
        pos, rgba, tris = scenes.grid_mesh(n, seed)
        m = max(2, int(round((n - 1) * math.sqrt(overlay_frac))) + 1)
        wpos, wrgba, wtris = scenes.water_mesh(m, water_level, water_alpha)
        dev = "cuda"
        self.layers = []
        for name, pp, cc, tt in (("terrain", pos, rgba, tris), ("water", wpos, wrgba, wtris)):
            self.layers.append({
                "name": name,
                "model": torch.from_numpy(np.ascontiguousarray(pp, dtype=np.float32)).to(dev),
                "colors": torch.from_numpy(np.ascontiguousarray(cc, dtype=np.float32)).to(dev),
                "indices": torch.from_numpy(np.ascontiguousarray(tt, dtype=np.int32)).to(dev),
                "num_tris": int(tt.shape[0]),
                "vbuf": [torch.empty((pp.shape[0], 8), dtype=torch.float32, device=dev)
                         for _ in range(1 if fused else self.VERTEX_SLOTS)],
            })
            if fused:   # static records: clip positions come from setup, colours stay
                vb = self.layers[-1]["vbuf"][0]
                vb[:, 0:4] = 0.0
                vb[:, 4:8] = self.layers[-1]["colors"]
                # Positions padded to 16 bytes: setup gathers each with one vector load.
                m4 = torch.ones((pp.shape[0], 4), dtype=torch.float32, device=dev)
                m4[:, 0:3] = self.layers[-1]["model"]
                self.layers[-1]["model4"] = m4
        self.targets = [(p.CudaSurface((width, height), p.CudaSurface.FORMAT_RGBA8, 1),
                         p.CudaSurface((width, height), p.CudaSurface.FORMAT_DEPTH32, 1)) for _ in range(self.TARGETS)]
        self.mvps = [scenes.terrain_camera(f, width, height).astype(np.float32) for f in range(frames)]
        self.num_tris = sum(layer["num_tris"] for layer in self.layers)

    def camera_delta(self, a: int, b: int) -> np.ndarray:
        return self.scenes.camera_delta(a, b)

    def contexts(self, tuning: dict | None = None):
        """One CudaRaster per layer (each keeps its own queues and counters)."""
        p = _pkg()
        out = []
        for k, layer in enumerate(self.layers):
            cr = p.CudaRaster()
            cr.init()
            if tuning:
                cr.setTuning(**tuning)
            cr.setSurfaces(*self.targets[0])
            cr.setPixelPipe(None, "PixelPipe_gouraud" if k == 0 else "PixelPipe_gouraud_srcover")
            cr.setIndexBuffer(layer["indices"], 0, layer["num_tris"])
            out.append(cr)
        return out

    def transform(self, frame: int, stream=None) -> None:
        if self.fused:
            return   # setup transforms the vertices of each draw (draw_layer)
        slot = frame % self.VERTEX_SLOTS
        for layer in self.layers:
            self.raster.vertex_shader_passthrough(layer["model"], self.mvps[frame], layer["colors"],
                                                  out=layer["vbuf"][slot], stream=stream)

    def draw_layer(self, cr, k: int, frame: int, stream, sync: bool = True) -> None:
        """Layer k of `frame` (0: opaque terrain with the deferred clear, 1:
        water) from the frame's vertex slot into its surface pair."""
        color, depth = self.target(frame)
        cr.setSurfaces(color, depth)
        layer = self.layers[k]
        if self.fused:
            cr.setVertexBuffer(layer["vbuf"][0], 0)
            cr.setVertexTransform(layer["model4"], self.mvps[frame])
        else:
            cr.setVertexBuffer(layer["vbuf"][frame % self.VERTEX_SLOTS], 0)
        if k == 0:
            cr.deferredClear(WATER_CLEAR[:4], WATER_CLEAR[4])
        if sync:
            cr.drawTriangles(stream)
        else:
            cr.drawTrianglesAsync(stream)

    def draw(self, crs, frame: int, stream, sync: bool = True) -> None:
        """Opaque terrain then the water layer of `frame`."""
        for k, cr in enumerate(crs):
            self.draw_layer(cr, k, frame, stream, sync)

    def target(self, frame: int):
        return self.targets[frame % self.TARGETS]

    def frame_plain(self, crs, frame: int, stream) -> None:
        self.transform(frame, stream)
        self.draw(crs, frame, stream, sync=True)

    def checksum(self, frame: int) -> int:
        """64-bit position-weighted sum of the colour and depth words of the
        surfaces `frame` was drawn into (enqueued on the current stream)."""
        color, depth = self.target(frame)
        if not hasattr(self, "_weights"):
            n = color.tensor.numel()
            idx = torch.arange(n, dtype=torch.int64, device="cuda")
            self._weights = (idx * 2654435761 + 12345) % 2147483647 + 1
        c = color.tensor.view(-1).to(torch.int64) & 0xFFFFFFFF
        d = depth.tensor.view(-1).to(torch.int64) & 0xFFFFFFFF
        return int(((c * self._weights).sum() + (d * self._weights.flip(0)).sum()).item())

    def snapshot(self, frame: int):
        color, depth = self.target(frame)
        return color.tensor.clone(), depth.tensor.clone()


def run_flythrough_plain(ft: FlyThrough, frames: range, tuning: dict | None = None, checksums: bool = False,
                         keep: tuple = ()):
    """The reference's usage: per frame, the vertex stage and two synchronous
    drawTriangles calls. Returns (wall seconds, per-frame checksums, kept
    frames, final counters)."""
    import time
    stream = torch.cuda.current_stream()
    crs = ft.contexts(tuning)
    sums, kept = [], {}
    torch.cuda.synchronize()
    wall = 0.0
    for f in frames:
        t0 = time.perf_counter()
        ft.frame_plain(crs, f, stream)
        torch.cuda.synchronize()
        wall += time.perf_counter() - t0
        if checksums:
            sums.append(ft.checksum(f))
        if f in keep:
            kept[f] = ft.snapshot(f)
    counters = [cr.getCounters() for cr in crs]
    return wall, sums, kept, counters


def run_flythrough_predicted(ft: FlyThrough, frames: int, train_frames: int = 50, tuning: dict | None = None,
                             checksums: bool = False, keep: tuple = (), train_steps: int = 4,
                             online_every: int = 4, seed: int = 0, lr: float = 3e-4, ahead: int = 2,
                             min_margin: float = 0.02, margin_factor: float = 2.0, capacity_scale: float = 1.0,
                             layer_streams: bool = True):
    """The first `train_frames` frames are plain (synchronous draws) and train
    one predictor per layer on the counts they emit. Later frames are drawn
    asynchronously into queues sized from predictions made `ahead` (= 2)
    frames earlier, so the host keeps one frame queued: at frame f it checks
    frame f - 2 (its overflow flags), then sizes and launches frame f. Each
    layer's predictor step runs on its own stream right after that layer's
    draw, and the next draw of the layer waits for it. A frame whose queues
    overflowed is redrawn through the plain overflow-detect-and-rerun path (on
    separate contexts, so the queued frame's counts survive) before its
    surfaces are reused, and the predictor steps are redone. capacity_scale
    (tests) scales the capacities given to the draws. With layer_streams each
    layer draws on its own stream, after the layer below it in the same frame:
    the layers have their own contexts and consecutive frames their own
    surfaces, so frame f's water layer may run beside frame f + 1's terrain.
    Returns wall times, misses and the per-frame record."""
    import time
    if ahead != 2:
        raise ValueError("the pipelined loop predicts two frames ahead")
    P = importlib.import_module(PKG + ".predictor")
    S = torch.cuda.current_stream()
    L = len(ft.layers)
    Q = [torch.cuda.Stream() for _ in range(L)]
    D = [S] + [torch.cuda.Stream() if layer_streams else S for _ in range(L - 1)]
    crs = ft.contexts(tuning)
    fallback = ft.contexts(tuning)
    preds = None
    R = ahead + 2
    ev_draw = [[torch.cuda.Event() for _ in range(R)] for _ in range(L)]
    ev_pred = [[torch.cuda.Event() for _ in range(R)] for _ in range(L)]
    sums, kept, rec, launched = {}, {}, [], {}
    wall_train, wall_pred, wait = 0.0, 0.0, 0.0
    misses = [0] * L
    extra = [0] * L             # most clip-generated subtriangles seen per layer

    def draw_and_step(cset, f, sync, prev=None):
        """Draw both layers of frame f; after each, its predictor step on its
        stream. prev: the frame whose step must finish before a layer's
        contexts are drawn again."""
        for k, cr in enumerate(cset):
            st = D[k]
            if prev is not None:
                st.wait_event(ev_pred[k][prev % R])
            if k > 0 and st is not D[k - 1]:
                st.wait_event(ev_draw[k - 1][f % R])    # a layer draws over the one below it
            ft.draw_layer(cr, k, f, st, sync)
            ev_draw[k][f % R].record(st)
            if preds is None:
                return
            Q[k].wait_event(ev_draw[k][f % R])
            preds[k].step(cr, f, ft.camera_delta(f, f + ahead), Q[k])
            ev_pred[k][f % R].record(Q[k])

    def present(f):
        if checksums:
            sums[f] = ft.checksum(f)
        if f in keep:
            kept[f] = ft.snapshot(f)

    def check_frame(f):
        """Frame f's steps have completed; redraw it if a queue overflowed."""
        ctr = [pr.counters_of(f) for pr in preds]
        missed = [int(c[5]) != 0 for c in ctr]
        if any(missed):
            for k, m in enumerate(missed):
                misses[k] += int(m)
            torch.cuda.synchronize()
            draw_and_step(fallback, f, True)        # the plain path: grows its queues and reruns until done
            if f + 1 in launched:
                for k, cr in enumerate(crs):        # frame f+1's trend used frame f's counts
                    preds[k].step(cr, f + 1, ft.camera_delta(f + 1, f + 1 + ahead), Q[k])
            torch.cuda.synchronize()
        for k, pr in enumerate(preds):
            c = pr.counters_of(f)
            extra[k] = max(extra[k], int(c[0]))
            if f in launched:
                pt, cb, ct, pb = launched[f][k]
                actual = (float(c[1]), float(c[3]))
                pr.score(pt, actual)
                rec.append({"frame": f, "layer": k, "pred_bin": pt[0], "pred_tile": pt[1], "perbin_bin": pb[0],
                            "perbin_tile": pb[1], "cap_bin": cb, "cap_tile": ct, "bin": actual[0],
                            "tile": actual[1], "miss": bool(missed[k])})
        present(f)

    torch.cuda.synchronize()
    ft.transform(0, S)
    for f in range(train_frames):
        # Plain frames, drawn on the contexts that later serve the reruns.
        t0 = time.perf_counter()
        if preds is None:
            ft.draw(fallback, f, S, sync=True)
            preds = [P.QueuePredictor(P.queue_layout(cr), ahead=ahead, seed=seed + k, lr=lr,
                                      min_margin=min_margin, margin_factor=margin_factor)
                     for k, cr in enumerate(fallback)]
            for k, cr in enumerate(fallback):
                preds[k].step(cr, f, ft.camera_delta(f, f + ahead), Q[k])
                ev_pred[k][f % R].record(Q[k])
        else:
            draw_and_step(fallback, f, True, prev=f - 1)
        ft.transform(f + 1, S)
        for k, pr in enumerate(preds):
            pr.train(train_steps, f, Q[k])
        torch.cuda.synchronize()
        wall_train += time.perf_counter() - t0
        for k, pr in enumerate(preds):
            extra[k] = max(extra[k], int(pr.counters_of(f)[0]))
        present(f)

    t0 = time.perf_counter()
    for f in range(train_frames, frames + ahead):
        j = f - ahead                    # the frame to check now
        tw = time.perf_counter()
        for k in range(L):
            ev_pred[k][j % R].synchronize()
        wait += time.perf_counter() - tw
        if j >= train_frames:
            check_frame(j)
        if f >= frames:
            continue
        caps = []
        for k, (pr, cr, layer) in enumerate(zip(preds, crs, ft.layers)):
            pt = pr.predicted_totals(f)
            cb, ct = (int(c * capacity_scale) for c in pr.capacity(pt))
            cr.setCapacity(layer["num_tris"] + max(4096, 2 * extra[k]), cb, ct)
            caps.append((pt, cb, ct, pr.per_bin_totals(f)))
        launched[f] = caps
        draw_and_step(crs, f, False, prev=f - 1)
        if f + 1 < frames:
            ft.transform(f + 1, S)
        if (f - train_frames) % online_every == 0:
            for k, pr in enumerate(preds):
                pr.train(1, j, Q[k])
    torch.cuda.synchronize()
    wall_pred = time.perf_counter() - t0
    steps = [pr.net.steps for pr in preds or []]
    for pr in preds or []:
        pr.close()
    return {"wall_train": wall_train, "wall_pred": wall_pred, "wait": wait, "misses": misses, "records": rec,
            "checksums": [sums[f] for f in sorted(sums)], "kept": kept, "train_frames": train_frames,
            "adam_steps": steps}


FLYTHROUGH_WORKLOAD = ("fly-through: 4096^2 heightfield (33.5M triangles, 6-octave value noise) + translucent water "
                       "layer (10% of the triangles, src-over) at 3840x2160, depth LESS, 300-frame camera loop; "
                       "per frame two draws with the vertex transform fused into setup; frames 0-49 plain and "
                       "training the predictor")


def measure_flythrough(n: int = 4096, width: int = 3840, height: int = 2160, frames: int = 300,
                       train_frames: int = 50, tuning: dict | None = None, keep: tuple = (), fused: bool = True):
    """Plain vs predictor-sized pipelined fly-through over the same frames.
    Returns (summary dict, {frame: (colour, depth)} of the plain pass, the
    FlyThrough)."""
    ft = FlyThrough(n=n, width=width, height=height, frames=frames, fused=fused)
    run_flythrough_plain(ft, range(3), tuning)                                   # warm-up
    _, sums, kept, ctr = run_flythrough_plain(ft, range(frames), tuning, checksums=True, keep=keep)
    exact = run_flythrough_predicted(ft, frames, train_frames, tuning, checksums=True)
    wall_plain, _, _, _ = run_flythrough_plain(ft, range(train_frames, frames), tuning)
    res = run_flythrough_predicted(ft, frames, train_frames, tuning)
    n_pred = frames - train_frames
    plain_fps = n_pred / wall_plain
    pred_fps = n_pred / res["wall_pred"]
    layers = []
    for k, layer in enumerate(ft.layers):
        r = sorted((x for x in res["records"] if x["layer"] == k), key=lambda x: x["frame"])
        T = layer["num_tris"]
        entry = {"layer": layer["name"], "triangles": T, "misses": res["misses"][k],
                 "queue_mb_plain_estimate": round((2 * T + 65536 + 4 * T + 65536) * 4 / 2**20, 1),
                 "queue_mb_predicted_mean": round(float(np.mean([x["cap_bin"] + x["cap_tile"] for x in r])) * 4 / 2**20,
                                                  1),
                 "queue_mb_predicted_max": round(float(np.max([x["cap_bin"] + x["cap_tile"] for x in r])) * 4 / 2**20,
                                                 1),
                 "queue_mb_used_max": round(float(np.max([x["bin"] + x["tile"] for x in r])) * 4 / 2**20, 1)}
        errs = {}
        for q in ("bin", "tile"):
            a = np.array([x[q] for x in r])
            p = np.array([x["pred_" + q] for x in r])
            # frame f is sized at frame f - 2: previous-frame sizing uses a[f-2],
            # trend extrapolation a[f-2] * (a[f-2] / a[f-3])^2.
            prev = a[1:-2]
            trend = a[1:-2] ** 3 / a[:-3] ** 2
            tgt = a[3:]
            errs[q] = {"predictor": round(float(np.abs(np.log(tgt / p[3:])).mean()), 5),
                       "previous_frame": round(float(np.abs(np.log(tgt / prev)).mean()), 5),
                       "trend_only": round(float(np.abs(np.log(tgt / trend)).mean()), 5),
                       "predictor_max": round(float(np.abs(np.log(tgt / p[3:])).max()), 5),
                       "previous_frame_max": round(float(np.abs(np.log(tgt / prev)).max()), 5)}
        entry["mean_abs_log_error"] = errs
        layers.append(entry)
    summary = {"workload": FLYTHROUGH_WORKLOAD, "frames": frames, "train_frames": train_frames,
               "triangles_per_frame": ft.num_tris, "plain_frames_per_s": round(plain_fps, 2),
               "predicted_frames_per_s": round(pred_fps, 2), "speedup": round(pred_fps / plain_fps, 3),
               "plain_mtri_per_s": round(ft.num_tris * plain_fps / 1e6, 1),
               "predicted_mtri_per_s": round(ft.num_tris * pred_fps / 1e6, 1),
               "bit_exact_vs_plain": exact["checksums"] == sums, "frames_checked": len(sums),
               "misses": res["misses"], "miss_rate": round(sum(res["misses"]) / (2 * n_pred), 4),
               "adam_steps": res["adam_steps"], "layers": layers,
               "plain": ("two synchronous drawTriangles per frame, vertex transform fused into setup" if fused
                         else "vertex stage + two synchronous drawTriangles per frame"),
               "predicted": "queues sized by the predictor two frames ahead, draws queued asynchronously, "
                            "one overflow check per frame, misses redrawn by the plain path"}
    return summary, kept, ft


SUBPIXEL_WORKLOAD = ("subpixel stress: 2048^2 heightfield (8.4M triangles, 6-octave value noise) at a grazing 15 deg "
                     "camera, 3840x2160, 4x MSAA, Gouraud, depth LESS, opaque; L2 flushed before each frame")


def measure_subpixel(n: int = 2048, width: int = 3840, height: int = 2160, samples: int = 4, frame: float = 120.0,
                     steps: int = 10, warmup: int = 3, tuning: dict | None = None):
    """Plain drawTriangles of the grazing-angle heightfield with 4x MSAA.
    Returns (summary, (colour, depth) tensors of the last frame, scene)."""
    p = _pkg()
    scenes = importlib.import_module(PKG + ".scenes")
    sc = scenes.terrain(n, width, height, samples, seed=5, frame=frame)
    T = int(sc["indices"].shape[0])
    cr = p.CudaRaster()
    cr.init()
    if tuning:
        cr.setTuning(**tuning)
    color = p.CudaSurface((width, height), p.CudaSurface.FORMAT_RGBA8, samples)
    depth = p.CudaSurface((width, height), p.CudaSurface.FORMAT_DEPTH32, samples)
    cr.setSurfaces(color, depth)
    cr.setPixelPipe(None, f"PixelPipe_gouraud_msaa{samples}")
    v = torch.from_numpy(sc["vertices"]).cuda()
    i = torch.from_numpy(np.ascontiguousarray(sc["indices"], dtype=np.int32)).cuda()
    cr.setVertexBuffer(v, 0)
    cr.setIndexBuffer(i, 0, T)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def draw():
        cr.deferredClear(CLEAR[:4], CLEAR[4])
        cr.drawTriangles(stream)

    for _ in range(warmup):
        draw()
    ms, stages = [], []
    for _ in range(steps):
        flush.fill_(1)
        ms += time_events(draw, 1, stream)
        st = cr.getStats()
        stages.append([st.setupTime, st.binTime, st.coarseTime, st.fineTime])
    c = cr.getCounters()
    med = float(np.median(ms))
    st_ms = np.median(np.array(stages), axis=0) * 1e3
    summary = {"workload": SUBPIXEL_WORKLOAD, "num_tris": T, "width": width, "height": height, "samples": samples,
               "frames_per_s": round(1000.0 / med, 2), "ms_per_frame": round(med, 4),
               "mtri_per_s": round(T / med / 1e3, 1),
               "stage_ms": {k: round(float(x), 4) for k, x in zip(("setup", "bin", "coarse", "fine"), st_ms)},
               "counters": {k: c[k] for k in ("num_subtris", "bin_entries", "tile_entries", "coarse_units",
                                              "reruns", "overflow")}}
    return summary, (color.tensor.clone(), depth.tensor.clone()), sc


def profile_frames(name: str, frames: int, tuning: dict | None = None) -> dict:
    """Draws a few frames of a workload and nothing else (for profiler runs):
    "subpixel" (the 4x MSAA heightfield), "flythrough" / "flythrough2048"
    (plain fly-through frames 100..100+frames over the 4096^2 or a 2048^2
    heightfield), "predicted" (a short predictor-sized fly-through: `frames`
    frames, the first two thirds plain and training) or "batch64" (`frames`
    replays of the uneven 64-scene batch's CUDA graph), "textured" (frames of
    the textured Phong heightfield: its vertex shader and one draw each) or
    "vertex" (`frames` launches of each vertex shader over 8M vertices)."""
    if name == "textured":
        s, _, _, _ = measure_textured(steps=frames, warmup=0, tuning=tuning)
        return {"profile": name, "frames": frames, "counters": s["counters"]}
    if name == "resolve":   # `frames` resolves of a 4x MSAA 3840x2160 colour surface
        p = _pkg()
        raster = importlib.import_module(PKG + ".raster")
        cs = p.CudaSurface((3840, 2160), p.CudaSurface.FORMAT_RGBA8, 4)
        g = torch.Generator(device="cuda").manual_seed(9)
        cs.tensor.copy_(torch.randint(-2**31, 2**31 - 1, cs.tensor.shape, generator=g, device="cuda",
                                      dtype=torch.int32))
        ms = time_events(lambda: cs.resolve(), max(frames, 1), torch.cuda.current_stream())
        return {"profile": name, "frames": frames, "ms": round(float(np.median(ms)), 4),
                "bytes_per_resolve": 3840 * 2160 * (16 + 4)}
    if name == "vertex":
        v = measure_vertex_shaders(n=8 << 20, steps=frames, warmup=0)   # 268 MB of input records, above L2
        return {"profile": name, "frames": frames, "vertices": v["vertices"]}
    if name == "batch64":
        p = _pkg()
        scenes = importlib.import_module(PKG + ".scenes")
        batch = Batch(scenes.batch(64, seed=4))
        cr = p.CudaRaster()
        cr.init()
        if tuning:
            cr.setTuning(**tuning)
        g = cr.createBatchGraph(batch.items)
        stream = torch.cuda.current_stream()
        for _ in range(frames):
            g.launch(stream)
        torch.cuda.synchronize()
        g.destroy()
        return {"profile": name, "frames": frames, "tris": batch.num_tris}
    if name == "subpixel":
        s, _, _ = measure_subpixel(steps=frames, warmup=0, tuning=tuning)
        return {"profile": name, "frames": frames, "counters": s["counters"]}
    ft = FlyThrough(n=2048 if name == "flythrough2048" else 4096, frames=max(frames, 3) + 100)
    if name in ("flythrough", "flythrough2048"):
        run_flythrough_plain(ft, range(100, 100 + frames), tuning)
        return {"profile": name, "frames": frames, "tris": ft.num_tris}
    if name == "predicted":
        res = run_flythrough_predicted(ft, frames, max(3, (2 * frames) // 3), tuning)
        return {"profile": name, "frames": frames, "misses": res["misses"], "adam_steps": res["adam_steps"]}
    raise ValueError(name)


TEXTURED_WORKLOAD = ("textured Phong: 2048^2 heightfield (8.4M triangles) as InputVertex records, four materials "
                     "(untextured, diffuse texture, diffuse + alpha-tested texture, second texture) from one "
                     "mip-mapped RGBA8 atlas, 3840x2160, 1 spp, depth LESS; per frame vertexShader_texPhong on the "
                     "GPU and one PixelPipe_texPhong draw; L2 flushed before each frame")


def measure_textured(n: int = 2048, width: int = 3840, height: int = 2160, frame: float = 120.0, steps: int = 10,
                     warmup: int = 3, tuning: dict | None = None):
    """The textured Phong pipe per frame: the texPhong vertex shader then one draw.
    Returns (summary, (colour, depth) tensors of the last frame, scene, shaded vertices)."""
    p = _pkg()
    scenes = importlib.import_module(PKG + ".scenes")
    raster = importlib.import_module(PKG + ".raster")
    sc = scenes.textured_terrain(n, width, height, seed=5, frame=frame)
    T = int(sc["indices"].shape[0])
    cr = p.CudaRaster()
    cr.init()
    if tuning:
        cr.setTuning(**tuning)
    color = p.CudaSurface((width, height), p.CudaSurface.FORMAT_RGBA8, 1)
    depth = p.CudaSurface((width, height), p.CudaSurface.FORMAT_DEPTH32, 1)
    cr.setSurfaces(color, depth)
    cr.setPixelPipe(None, "PixelPipe_texPhong")
    inp = torch.from_numpy(sc["input"]).cuda()
    shaded = torch.empty((inp.shape[0], 16), dtype=torch.float32, device="cuda")
    mats = torch.from_numpy(sc["materials"]).cuda()
    tri = torch.from_numpy(sc["triangle_material_idx"]).cuda()
    atlas = torch.from_numpy(sc["atlas"].view(np.int32)).cuda()
    raster.set_tex_phong_constants(mats, tri, atlas)
    i = torch.from_numpy(np.ascontiguousarray(sc["indices"], dtype=np.int32)).cuda()
    cr.setVertexBuffer(shaded, 0)
    cr.setIndexBuffer(i, 0, T)
    k = (sc["pos_to_clip"], sc["pos_to_camera"], sc["normal_to_camera"])
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def frame_fn():
        raster.vertex_shader_tex_phong(inp, *k, out=shaded, stream=stream)
        cr.deferredClear(CLEAR[:4], CLEAR[4])
        cr.drawTriangles(stream)

    for _ in range(warmup):
        frame_fn()
    ms, stages = [], []
    for _ in range(steps):
        flush.fill_(1)
        ms += time_events(frame_fn, 1, stream)
        st = cr.getStats()
        stages.append([st.setupTime, st.binTime, st.coarseTime, st.fineTime])
    c = cr.getCounters()
    med = float(np.median(ms))
    st_ms = np.median(np.array(stages), axis=0) * 1e3
    summary = {"workload": TEXTURED_WORKLOAD, "num_tris": T, "num_vertices": int(inp.shape[0]), "width": width,
               "height": height, "frames_per_s": round(1000.0 / med, 2), "ms_per_frame": round(med, 4),
               "mtri_per_s": round(T / med / 1e3, 1),
               "stage_ms": {"setup": round(st_ms[0], 4), "bin": round(st_ms[1], 4), "coarse": round(st_ms[2], 4),
                            "fine": round(st_ms[3], 4)},
               "counters": {key: c[key] for key in ("num_subtris", "bin_entries", "tile_entries", "reruns",
                                                    "overflow")}}
    return summary, (color.tensor, depth.tensor), sc, shaded


def measure_vertex_shaders(n: int = 4096 * 4096, steps: int = 10, warmup: int = 3, peak_gbs: float | None = None):
    """The vertex shaders over n vertices (inputs far larger than L2, so no flush is
    needed): median time per launch, vertices/s and algorithmic bytes per second --
    passthrough 12 B position + 16 B colour in, 32 B out; Gouraud 32 B InputVertex +
    4 B material index in, 32 B out (the material table stays cached); texPhong 32 B
    in, 64 B out."""
    raster = importlib.import_module(PKG + ".raster")
    scenes = importlib.import_module(PKG + ".scenes")
    g = torch.Generator(device="cuda").manual_seed(3)
    inp = torch.rand((n, 8), generator=g, device="cuda", dtype=torch.float32) * 2.0 - 1.0
    model = inp[:, 0:3].contiguous()
    colors = torch.rand((n, 4), generator=g, device="cuda", dtype=torch.float32)
    midx = torch.randint(0, 4, (n,), generator=g, device="cuda", dtype=torch.int32)
    mats = torch.from_numpy(raster.material_records([[0.7, 0.6, 0.5, 1.0]] * 4, [[0.3, 0.3, 0.3]] * 4,
                                                    [8.0, 16.0, 32.0, 64.0])).cuda()
    view = scenes.look_at((1.5, 2.0, 3.0), (0.0, 0.0, 0.0)).astype(np.float32)
    clip = (scenes.perspective(60.0, 16 / 9, 0.1, 100.0) @ view).astype(np.float32)
    normal = view[:3, :3].copy()
    out8 = torch.empty((n, 8), dtype=torch.float32, device="cuda")
    out16 = torch.empty((n, 16), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    shaders = {
        "passthrough": (lambda: raster.vertex_shader_passthrough(model, clip, colors, out=out8, stream=stream),
                        12 + 16 + 32),
        "gouraud": (lambda: raster.vertex_shader_gouraud(inp, clip, view, normal, mats, midx, out=out8,
                                                         stream=stream), 32 + 4 + 32),
        "tex_phong": (lambda: raster.vertex_shader_tex_phong(inp, clip, view, normal, out=out16, stream=stream),
                      32 + 64),
    }
    res = {}
    for name, (fn, per_vertex) in shaders.items():
        for _ in range(warmup):
            fn()
        med = float(np.median(time_events(fn, steps, stream)))
        gbs = n * per_vertex / (med * 1e-3) / 1e9
        res[name] = {"ms": round(med, 4), "gvertices_per_s": round(n / med / 1e6, 2),
                     "alg_bytes_per_vertex": per_vertex, "achieved_gbs": round(gbs, 1)}
        if peak_gbs:
            res[name]["frac_of_measured_hbm"] = round(gbs / peak_gbs, 4)
    return {"workload": f"{n:,} vertices (random InputVertex records), each shader timed alone", "vertices": n,
            "shaders": res}
