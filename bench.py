"""Benchmark of the GB300 rasterizer on the plain-path-at-scale configuration:
a 1M-triangle random soup at 1920x1080, 1 sample per pixel, Gouraud shading,
depth LESS, opaque (seeded synthetic input).

One step = one drawTriangles() of the whole soup through the C ABI (the
reference's plain path: setup -> bin -> coarse -> fine, then the host reads
the overflow counters). `value` is device-timed with CUDA events on the
drawing stream, inputs resident in HBM, L2 flushed (256 MiB write) before
every step, per-stage timing events off; a second, shorter pass with them on
gives the stage times the roofline uses. `e2e` times the same draw with the inputs copied from pinned host
memory and the framebuffer copied back inside the timed region (wall clock over
all steps; the next step's inputs upload and the previous step's framebuffer
downloads on their own streams while the current step draws).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Two sub-objects compare the plain single-scene path with the batched and the
predictor-sized paths, bit for bit: "batched" (64 uneven scenes drawn one by
one vs one CUDA-graph replay of all of them) and "flythrough" (a 300-frame
camera loop over a 4096^2 heightfield plus a translucent water layer at
3840x2160: synchronous plain draws vs draws sized two frames ahead by the
learned queue predictor and queued asynchronously).

With --impl reference the CPU restatement of the reference pipeline (the
oracle, OpenMP over all host cores) renders the same scene; under torchrun
only rank 0 runs it.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
PKG = "cudaraster-linux_gb300"

# The library's kernels in one blocking draw of the soup: the draw-block write,
# setup, bin count / scan / scatter, coarse count / scan / scatter and fine.
KERNELS_PER_DRAW = 9
METRIC = "frames/s & Mtri/s on 1 GB300: batched+predicted vs plain, bit-exact framebuffers"
WORKLOAD = {"workload": "plain path at scale: 1M-triangle random soup, 1920x1080, 1 spp, Gouraud, depth LESS, opaque",
            "num_tris": 1_000_000, "width": 1920, "height": 1080, "samples": 1, "pipe": "PixelPipe_gouraud",
            "seed": 2, "l2": "flushed before every step (256 MiB write)"}


def scenes_module():
    """The seeded scene generator (pure numpy), loaded from its file without importing the
    package, so the reference arm maps none of the product's native code."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("cr_bench_scenes", ROOT / PKG / "scenes.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def load_scene():
    return scenes_module().soup(WORKLOAD["num_tris"], WORKLOAD["width"], WORKLOAD["height"], seed=WORKLOAD["seed"])


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def stage_traffic(stage: str):
    """DRAM bytes (read + write) of one launch of a stage's kernels on this
    workload, from the committed ncu summary of the same command, or None."""
    p = ROOT / "profiles" / "stages_soup1m_1080p.traffic.json"
    if not p.exists():
        return None
    return json.loads(p.read_text())["dram_bytes_per_stage"].get(stage)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 20 ms from before
    the timed region starts; mark() brackets the timed region and summary()
    keeps the samples nvidia-smi timestamped inside it."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, interval_ms: int = 20):
        self.gpu = gpu_index
        self.interval = interval_ms
        self.proc = None
        self.lines: list[str] = []
        self.window = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)  # let the first samples arrive
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def mark(self, start: float, end: float) -> None:
        self.window = (start, end)

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(2 * self.interval / 1000.0)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        import datetime
        sm, mx, reasons, kept = [], 0.0, set(), 0
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                continue
            if self.window and not (self.window[0] - 0.01 <= ts <= self.window[1] + 0.01):
                continue
            try:
                sm.append(float(parts[2]))
                mx = max(mx, float(parts[3]))
            except ValueError:
                continue
            kept += 1
            for n, v in zip(names, parts[6:10]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": kept, "interval_ms": self.interval}


def cpu_baseline(sc, budget_s: float = 12.0, min_frames: int = 1):
    """The oracle (CPU restatement of the reference pipeline, OpenMP) on the same scene."""
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    pipe = orc.make_pipe(sc["width"], sc["height"], 1, orc.DEPTH | orc.LERP, "replace", "gouraud",
                         clear=orc.clear_values((0.2, 0.4, 0.8, 1.0), 1.0))
    frames, t0, out = 0, time.perf_counter(), None
    while True:
        out = orc.render(pipe, sc["vertices"], sc["indices"], threads=threads)
        frames += 1
        if frames >= min_frames and time.perf_counter() - t0 >= budget_s:
            break
    el = time.perf_counter() - t0
    return {"value": frames / el, "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"{frames} full frame(s) of the same 1M-triangle scene in {el:.1f} s",
            "mtri_per_s": frames * sc["indices"].shape[0] / el / 1e6}, out


def reduce_max(x: float, world: int, device="cuda") -> float:
    """The largest x over the ranks (one all-reduce; x itself for one rank)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, steps: int, total_ms: float) -> float:
    """Frames per second of N independent replicas that each drew `steps`
    frames, the slowest in `total_ms` (weak scaling: work grows with N)."""
    return world * steps / (total_ms / 1e3)


def run_reference(args, rank, world):
    if rank != 0:
        return
    sc = load_scene()
    steps = max(1, args.steps)
    # Each step renders one whole frame (about 0.12 s on 16 Grace cores), so
    # the run's warm-up frames and timed frames are the ones asked for.
    for _ in range(max(0, args.warmup)):
        cpu_baseline(sc, budget_s=0.0)
    cb, _ = cpu_baseline(sc, budget_s=0.0, min_frames=steps)
    line = {"impl": "reference", "metric": METRIC, "value": round(cb["value"], 4), "unit": "frames/s",
            "n_gpus": world, "steps": steps, "warmup": args.warmup, "ms_per_step": round(1000.0 / cb["value"], 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+int32",
            "data": "synthetic (seeded)", "config": WORKLOAD, "mtri_per_s": round(cb["mtri_per_s"], 3),
            "cpu_baseline": cb, "e2e": {"value": round(cb["value"], 4), "unit": "frames/s",
                                         "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


FLY_ORACLE_FRAME = 150


def flythrough_oracle_check(ft, kept, f):
    """One fly-through frame of the plain pass against the CPU oracle (both
    layers, all host cores)."""
    import time
    from oracle import oracle as orc
    from oracle import vertex_oracle
    pkg = importlib.import_module(PKG)
    workloads = importlib.import_module(PKG + ".workloads")
    t0 = time.perf_counter()
    clear = (pkg.color_to_abgr(*workloads.WATER_CLEAR[:4]), pkg.clear_depth_from_float(workloads.WATER_CLEAR[4]))
    color = depth = None
    for k, layer in enumerate(ft.layers):
        clip = vertex_oracle.vertex_passthrough(layer["model"].cpu().numpy(), ft.mvps[f])
        verts = np.concatenate([clip, layer["colors"].cpu().numpy()], axis=1).astype(np.float32)
        p = orc.make_pipe(ft.width, ft.height, 1, orc.DEPTH | orc.LERP, "replace" if k == 0 else "srcover",
                          "gouraud", 32, clear if k == 0 else None)
        color, depth, _ = orc.render(p, verts, layer["indices"].cpu().numpy(), color, depth, 0)
    gc = kept[f][0].cpu().numpy().view(np.uint32)
    gd = kept[f][1].cpu().numpy().view(np.uint32)
    return {"frame": f, "bit_exact": bool((gc == color).all() and (gd == depth).all()),
            "oracle_s": round(time.perf_counter() - t0, 1)}


def textured_oracle_check(tex):
    """The textured frame against the CPU oracle: the GPU's shaded vertices against the
    vertex oracle, then the frame (all host cores)."""
    import time
    from oracle import oracle as orc
    from oracle import vertex_oracle
    pkg = importlib.import_module(PKG)
    workloads = importlib.import_module(PKG + ".workloads")
    _, (color, depth), sc, shaded = tex
    t0 = time.perf_counter()
    k = (sc["pos_to_clip"], sc["pos_to_camera"], sc["normal_to_camera"])
    verts = vertex_oracle.vertex_tex_phong(sc["input"], *k)
    vertex_exact = bool(np.array_equal(verts.view(np.uint32), shaded.cpu().numpy().view(np.uint32)))
    orc.set_tex_phong(sc["materials"], sc["triangle_material_idx"], sc["atlas"])
    clear = (pkg.color_to_abgr(*workloads.CLEAR[:4]), pkg.clear_depth_from_float(workloads.CLEAR[4]))
    p = orc.make_pipe(sc["width"], sc["height"], 1, orc.DEPTH | orc.LERP, "replace", "texphong", 64, clear)
    rc, rd, st = orc.render(p, verts, sc["indices"], None, None, 0)
    gc = color.cpu().numpy().view(np.uint32)
    gd = depth.cpu().numpy().view(np.uint32)
    return {"vertices_bit_exact": vertex_exact, "bit_exact": bool((gc == rc).all() and (gd == rd).all()),
            "zmin_violations": int(st["zmin_violations"]), "oracle_s": round(time.perf_counter() - t0, 1)}


def subpixel_oracle_check(sc, got):
    """The 4x MSAA heightfield frame against the CPU oracle (all host cores)."""
    import time
    from oracle import oracle as orc
    pkg = importlib.import_module(PKG)
    workloads = importlib.import_module(PKG + ".workloads")
    t0 = time.perf_counter()
    clear = (pkg.color_to_abgr(*workloads.CLEAR[:4]), pkg.clear_depth_from_float(workloads.CLEAR[4]))
    p = orc.make_pipe(sc["width"], sc["height"], sc["samples"], orc.DEPTH | orc.LERP, "replace", "gouraud", 32, clear)
    rc, rd, st = orc.render(p, sc["vertices"], sc["indices"], None, None, 0)
    gc = got[0].cpu().numpy().view(np.uint32)
    gd = got[1].cpu().numpy().view(np.uint32)
    return {"bit_exact": bool((gc == rc).all() and (gd == rd).all()), "zmin_violations": st["zmin_violations"],
            "oracle_s": round(time.perf_counter() - t0, 1)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the uneven-batch comparison")
    ap.add_argument("--no-flythrough", action="store_true", help="skip the fly-through with the queue predictor")
    ap.add_argument("--no-subpixel", action="store_true", help="skip the 4x MSAA grazing-heightfield frame")
    ap.add_argument("--no-textured", action="store_true",
                    help="skip the textured Phong frame and the vertex-shader throughput lines")
    ap.add_argument("--profile-frames", type=int, default=0,
                    help="only draw this many frames of the workload (for ncu captures), print nothing else")
    ap.add_argument("--profile-workload", default="soup1m", choices=["soup1m", "subpixel", "flythrough", "flythrough2048",
                                                              "predicted", "batch64", "textured", "vertex", "resolve"],
                    help="workload of --profile-frames: the 1M soup (default), the 4x MSAA heightfield, plain "
                         "fly-through frames, predictor-sized fly-through frames (12 of them, 8 training), "
                         "replays of the uneven 64-scene batch, textured Phong frames, vertex-shader launches or "
                         "MSAA resolves of a 4x 4K surface")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    pkg = importlib.import_module(PKG)
    sc = load_scene()
    T = sc["indices"].shape[0]
    W, H = sc["width"], sc["height"]

    workloads = importlib.import_module(PKG + ".workloads")
    tuning = workloads.load_tuning("soup1m")
    if args.profile_frames > 0 and args.profile_workload != "soup1m":
        wname = "flythrough" if args.profile_workload.startswith("flythrough") or args.profile_workload == "predicted" \
            else {"textured": "subpixel", "vertex": "soup1m", "resolve": "soup1m"}.get(args.profile_workload,
                                                                                     args.profile_workload)
        print(json.dumps(workloads.profile_frames(args.profile_workload, args.profile_frames,
                                                  workloads.load_tuning(wname))))
        return
    cr = pkg.CudaRaster()
    cr.init()
    if tuning:
        cr.setTuning(**tuning)
    color = pkg.CudaSurface((W, H), pkg.CudaSurface.FORMAT_RGBA8, 1)
    depth = pkg.CudaSurface((W, H), pkg.CudaSurface.FORMAT_DEPTH32, 1)
    cr.setSurfaces(color, depth)
    cr.setPixelPipe(None, WORKLOAD["pipe"])
    verts = torch.from_numpy(sc["vertices"]).cuda()
    idx = torch.from_numpy(sc["indices"]).cuda()
    cr.setVertexBuffer(verts, 0)
    cr.setIndexBuffer(idx, 0, T)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def draw():
        cr.deferredClear((0.2, 0.4, 0.8, 1.0), 1.0)
        cr.drawTriangles(stream)

    if args.profile_frames > 0:
        cr.setStageTiming(False)
        for _ in range(args.profile_frames):
            draw()
        torch.cuda.synchronize()
        print(json.dumps({"profile_frames": args.profile_frames, "counters": cr.getCounters()}))
        return

    for _ in range(max(3, args.warmup)):
        draw()
    torch.cuda.synchronize()

    # ---- device-timed steps. The headline pass draws without the per-stage
    # events of getStats (they separate the stage kernels' launches); a second
    # pass with them on gives the stage times of the roofline.
    def timed(n, stage_timing):
        cr.setStageTiming(stage_timing)
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(n)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(n)]
        stage = np.zeros(4)
        for i in range(n):
            flush.fill_(i & 0xFF)
            starts[i].record(stream)
            draw()
            ends[i].record(stream)
            if stage_timing:
                s = cr.getStats()
                stage += [s.setupTime, s.binTime, s.coarseTime, s.fineTime]
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in zip(starts, ends)), stage / n * 1e3

    stage_steps = max(1, min(args.steps, 100))
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_start = time.time()
        total_ms, _ = timed(args.steps, False)
        staged_ms, stage_ms = timed(stage_steps, True)
        clk.mark(t_start, time.time())
    if world > 1:
        dist.barrier()
    total_ms = reduce_max(total_ms, world, "cuda")
    ms_per_step = total_ms / args.steps
    value = replica_throughput(world, args.steps, total_ms)
    counters = cr.getCounters()

    # ---- end-to-end through the C ABI with host buffers: every step copies its
    # vertex and index buffers in from pinned host memory and its framebuffer
    # out. Three input sets (uploaded two steps ahead on a copy stream, so the
    # link always has a copy queued) and two framebuffers (the previous step's
    # downloads on a readback stream) rotate while step i draws.
    hv = torch.from_numpy(sc["vertices"]).pin_memory()
    hi = torch.from_numpy(sc["indices"]).pin_memory()
    hc = [torch.empty_like(color.tensor, device="cpu").pin_memory() for _ in range(2)]
    hd = [torch.empty_like(depth.tensor, device="cpu").pin_memory() for _ in range(2)]
    NIN = 3
    dev_in = [(torch.empty_like(verts), torch.empty_like(idx)) for _ in range(NIN)]
    fbs = [(color, depth), (pkg.CudaSurface((W, H), pkg.CudaSurface.FORMAT_RGBA8, 1),
                            pkg.CudaSurface((W, H), pkg.CudaSurface.FORMAT_DEPTH32, 1))]
    up_stream, down_stream = torch.cuda.Stream(), torch.cuda.Stream()
    copied = [torch.cuda.Event() for _ in range(NIN)]
    drawn = [torch.cuda.Event() for _ in range(NIN)]
    read = [torch.cuda.Event() for _ in range(2)]

    def upload(k):
        up_stream.wait_event(drawn[k % NIN])       # the draw that read this input set is done
        with torch.cuda.stream(up_stream):
            dev_in[k % NIN][0].copy_(hv, non_blocking=True)
            dev_in[k % NIN][1].copy_(hi, non_blocking=True)
        copied[k % NIN].record(up_stream)

    def e2e_run(n):
        for k in range(min(NIN - 1, n)):
            upload(k)
        for k in range(n):
            if k + NIN - 1 < n:
                upload(k + NIN - 1)
            stream.wait_event(copied[k % NIN])
            stream.wait_event(read[k % 2])          # this framebuffer's previous readback is done
            dv, di = dev_in[k % NIN]
            cr.setSurfaces(*fbs[k % 2])
            cr.setVertexBuffer(dv, 0)
            cr.setIndexBuffer(di, 0, T)
            draw()
            drawn[k % NIN].record(stream)
            down_stream.wait_event(drawn[k % NIN])
            with torch.cuda.stream(down_stream):
                hc[k % 2].copy_(fbs[k % 2][0].tensor, non_blocking=True)
                hd[k % 2].copy_(fbs[k % 2][1].tensor, non_blocking=True)
            read[k % 2].record(down_stream)
        torch.cuda.synchronize()

    e2e_run(3)
    t0 = time.perf_counter()
    e2e_run(args.steps)
    e2e_total = (time.perf_counter() - t0) * 1e3
    e2e_total = reduce_max(e2e_total, world, "cuda")
    e2e_value = replica_throughput(world, args.steps, e2e_total)
    cr.setSurfaces(color, depth)
    h2d = hv.numel() * 4 + hi.numel() * 4
    d2h = (hc[0].numel() + hd[0].numel()) * 4

    # ---- roofline of the dominant stage (stage events bracket its kernels)
    peak, peak_kind = peaks()
    names = ["setup", "bin", "coarse", "fine"]
    dom = int(np.argmax(stage_ms))
    V = sc["vertices"].shape[0]
    # Algorithmic bytes per launch of each stage (one frame), each byte counted once:
    #   setup : index 12 B per triangle, each clip position 16 B once; subtri byte + header 16 B + data 64 B written
    #   bin   : subtri byte + header per triangle read, 4 B per bin entry written
    #   coarse: 4 B entry + 16 B header per bin entry read, 4 B per tile entry written
    #   fine  : 4 B per tile entry, header + data once per bin entry, colour + depth of every sample written
    N = ((W + 7) // 8 * 8) * ((H + 7) // 8 * 8)
    alg = {
        "setup": T * (12 + 1 + 16 + 64) + V * 16,
        "bin": T * 17 + counters["bin_entries"] * 4,
        "coarse": counters["bin_entries"] * 20 + counters["tile_entries"] * 4,
        "fine": counters["tile_entries"] * 4 + counters["bin_entries"] * 80 + N * 8,
    }
    achieved = alg[names[dom]] / (stage_ms[dom] / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": names[dom], "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                "traffic": stage_traffic(names[dom]), "alg_bytes_per_launch": int(alg[names[dom]]),
                "stage_ms": {n: round(float(m), 4) for n, m in zip(names, stage_ms)}}
    b_alg = 12 * T + 32 * V + 8 * N
    frame_frac = b_alg / (ms_per_step / 1e3) / 1e9 / peak

    line = {"metric": METRIC, "value": round(value, 3), "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+int32", "data": "synthetic (seeded)",
            "config": WORKLOAD, "mtri_per_s": round(T * value / 1e6, 2),
            "frame_roofline_frac": round(frame_frac, 4), "frame_alg_bytes": int(b_alg),
            "e2e": {"value": round(e2e_value, 3), "unit": "frames/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_total / args.steps, 4)},
            "roofline": roofline, "clocks": clk.summary(),
            "ms_per_step_with_stage_events": round(staged_ms / stage_steps, 4),
            "gpu_launches": KERNELS_PER_DRAW * args.steps, "counters": counters, "tuning": tuning}
    if not args.no_batch:
        scenes = importlib.import_module(PKG + ".scenes")
        batch = workloads.Batch(scenes.batch(64, seed=4))
        line["batched"] = dict(workloads.measure_batch(batch, steps=5, tuning=workloads.load_tuning("batch64")),
                               workload="uneven batch: 64 random soups, 1k-500k triangles (log-uniform), "
                                        "resolutions 256^2..1920x1080, half src-over blended; "
                                        "plain = 64 sequential drawTriangles, batched = one CUDA-graph replay")
    sub = None
    if rank == 0 and not args.no_subpixel:
        sub = workloads.measure_subpixel(tuning=workloads.load_tuning("subpixel"))
        line["subpixel_stress"] = sub[0]
    tex = None
    if rank == 0 and not args.no_textured:
        tex = workloads.measure_textured(tuning=workloads.load_tuning("subpixel"))
        line["textured"] = tex[0]
        line["vertex_shaders"] = workloads.measure_vertex_shaders(peak_gbs=peaks()[0])
    fly = None
    if rank == 0 and not args.no_flythrough:
        fly = workloads.measure_flythrough(tuning=workloads.load_tuning("flythrough"), keep=(FLY_ORACLE_FRAME,))
        line["flythrough"] = fly[0]
    if rank == 0 and not args.no_cpu_baseline:
        cb, (rc, rd, st) = cpu_baseline(sc)
        gc = color.download().numpy().astype(np.uint32)
        gd = depth.download().numpy().astype(np.uint32)
        line["cpu_baseline"] = cb
        line["bit_exact_vs_oracle"] = bool((gc == rc).all() and (gd == rd).all())
        if fly is not None:
            line["flythrough"]["oracle_frame"] = flythrough_oracle_check(fly[2], fly[1], FLY_ORACLE_FRAME)
        if sub is not None:
            line["subpixel_stress"]["oracle"] = subpixel_oracle_check(sub[2], sub[1])
        if tex is not None:
            line["textured"]["oracle"] = textured_oracle_check(tex)
    if rank == 0:
        # The full record first (a text-prefixed line, not JSON), then the
        # headline JSON line last and short: every config's speed and
        # bit-exactness stay in a reader's last few kilobytes of output.
        print("bench detail: " + json.dumps(line), flush=True)
        print(json.dumps(headline(line)), flush=True)
    if world > 1:
        dist.destroy_process_group()


def headline(line: dict) -> dict:
    """The contract's keys plus, per configuration, only its speed, its
    comparison and its bit-exactness flags."""
    keep = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "config", "mtri_per_s", "frame_roofline_frac", "e2e", "clocks",
            "gpu_launches", "bit_exact_vs_oracle")
    out = {k: line[k] for k in keep if k in line}
    r = line["roofline"]
    out["roofline"] = {k: r[k] for k in ("bound", "kernel", "achieved", "peak", "unit", "frac", "traffic",
                                         "alg_bytes_per_launch", "peak_kind")}
    if "cpu_baseline" in line:
        cb = line["cpu_baseline"]
        out["cpu_baseline"] = {k: (round(cb[k], 3) if isinstance(cb[k], float) else cb[k])
                               for k in ("value", "unit", "cores", "kind", "sample")}
    if "subpixel_stress" in line:
        s = line["subpixel_stress"]
        o = s.get("oracle", {})
        out["subpixel_stress"] = {"frames_per_s": s["frames_per_s"], "mtri_per_s": s["mtri_per_s"],
                                  "bit_exact_vs_oracle": o.get("bit_exact"),
                                  "zmin_violations": o.get("zmin_violations")}
    if "batched" in line:
        b = line["batched"]
        out["batched"] = {"plain_frames_per_s": b["plain_frames_per_s"],
                          "batched_frames_per_s": b["batched_frames_per_s"], "speedup": b["speedup"],
                          "bit_exact_vs_plain": b["bit_exact_vs_plain"], "scenes": b["scenes"]}
    if "flythrough" in line:
        f = line["flythrough"]
        o = f.get("oracle_frame", {})
        out["flythrough"] = {"plain_frames_per_s": f["plain_frames_per_s"],
                             "predicted_frames_per_s": f["predicted_frames_per_s"], "speedup": f["speedup"],
                             "bit_exact_vs_plain": f["bit_exact_vs_plain"], "frames_checked": f["frames_checked"],
                             "oracle_frame": o.get("frame"), "oracle_frame_bit_exact": o.get("bit_exact"),
                             "miss_rate": f["miss_rate"]}
        for k in ("culled_frames_per_s", "predictor_vs_trend"):
            if k in f:
                out["flythrough"][k] = f[k]
    if "textured" in line:
        t = line["textured"]
        o = t.get("oracle", {})
        out["textured"] = {"frames_per_s": t["frames_per_s"], "bit_exact_vs_oracle": o.get("bit_exact"),
                           "vertices_bit_exact": o.get("vertices_bit_exact")}
    if "vertex_shaders" in line:
        out["vertex_shaders_frac_of_hbm"] = {k: v.get("frac_of_measured_hbm")
                                             for k, v in line["vertex_shaders"]["shaders"].items()}
    return out


if __name__ == "__main__":
    main()
