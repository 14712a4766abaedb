"""Learned queue-occupancy predictor.

`Network` wraps the native MLP (cr_predictor_*: BF16 parameters, FP32
accumulation, Adam; kernels in csrc/predictor.cu). `QueuePredictor` runs it
online beside one draw stream: after each frame it takes the per-bin and
per-tile queue counts the rasterizer emitted (cr_queue_counts), trains on the
pair (previous frame's histogram + camera delta -> this frame's occupancy),
and predicts the next frame's bin- and tile-queue occupancy, from which the
queue capacities of the next draw are set (CudaRaster.setCapacity). A draw
whose queues overflow anyway is redrawn by the plain overflow-detect-and-
rerun path, which also catches and redraws the predictor's misses.

The reference has no learned part: it sizes its queues from the previous
draw and grows them on overflow (src/cudaraster/CudaRaster.cpp:263-275,
325-342).
"""
from __future__ import annotations

import ctypes as C
import math
from collections import deque

import numpy as np
import torch

from . import _lib

HIST_INPUTS = 16 * 16 + 6


def init_params(dims, seed: int = 0) -> np.ndarray:
    """Weights uniform in +-1/sqrt(fan_in), zero biases and a zero output
    layer, so an untrained network predicts "same occupancy as last frame"."""
    inputs, h1, h2, outputs = dims
    rng = np.random.default_rng(seed)
    parts = [rng.uniform(-1, 1, (h1, inputs)) / math.sqrt(inputs), np.zeros(h1),
             rng.uniform(-1, 1, (h2, h1)) / math.sqrt(h1), np.zeros(h2),
             np.zeros((outputs, h2)), np.zeros(outputs)]
    return np.concatenate([p.reshape(-1) for p in parts]).astype(np.float32)


def _p(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def _s(stream) -> int | None:
    return (stream or torch.cuda.current_stream()).cuda_stream


class Network:
    """inputs -> hidden1 -> hidden2 -> outputs MLP on the GPU."""

    def __init__(self, inputs: int, hidden1: int = 64, hidden2: int = 64, outputs: int = 1,
                 max_batch: int = 64, seed: int = 0, params: np.ndarray | None = None):
        self.lib = _lib.load()
        self.dims = (inputs, hidden1, hidden2, outputs)
        self.max_batch = max_batch
        h = C.c_void_p()
        _lib.check(self.lib.cr_predictor_create(C.byref(h), inputs, hidden1, hidden2, outputs, max_batch))
        self.handle = h
        self.num_params = int(self.lib.cr_predictor_num_params(h))
        self.set_params(init_params(self.dims, seed) if params is None else params)
        self._loss = torch.zeros(1, dtype=torch.float32, device="cuda")

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.cr_predictor_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def steps(self) -> int:
        return int(self.lib.cr_predictor_steps(self.handle))

    def set_params(self, params: np.ndarray) -> None:
        a = np.ascontiguousarray(params, dtype=np.float32)
        if a.size != self.num_params:
            raise ValueError(f"expected {self.num_params} parameters, got {a.size}")
        _lib.check(self.lib.cr_predictor_set_params(self.handle, a.ctypes.data_as(C.POINTER(C.c_float)), a.size))

    def get_params(self) -> np.ndarray:
        a = np.empty(self.num_params, np.float32)
        _lib.check(self.lib.cr_predictor_get_params(self.handle, a.ctypes.data_as(C.POINTER(C.c_float)), a.size))
        return a

    def get_params_bf16(self) -> np.ndarray:
        """The BF16 parameters the kernels use, as float32 values."""
        a = np.empty(self.num_params, np.uint16)
        _lib.check(self.lib.cr_predictor_get_params_bf16(self.handle, a.ctypes.data_as(C.POINTER(C.c_uint16)),
                                                         a.size))
        return (a.astype(np.uint32) << 16).view(np.float32)

    def forward(self, x: torch.Tensor, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        x = x.contiguous()
        b = x.shape[0]
        if out is None:
            out = torch.empty((b, self.dims[3]), dtype=torch.float32, device=x.device)
        _lib.check(self.lib.cr_predictor_forward(self.handle, _p(x), b, _p(out), _s(stream)))
        return out

    def gradients(self, x_pool: torch.Tensor, t_pool: torch.Tensor, rows: torch.Tensor | None = None,
                  batch: int | None = None, stream=None):
        batch = batch or (rows.shape[0] if rows is not None else x_pool.shape[0])
        s = stream or torch.cuda.current_stream()
        with torch.cuda.stream(s):
            g = torch.empty(self.num_params, dtype=torch.float32, device=x_pool.device)
            loss = torch.empty(1, dtype=torch.float32, device=x_pool.device)
        _lib.check(self.lib.cr_predictor_gradients(self.handle, _p(x_pool), _p(t_pool), x_pool.shape[0], _p(rows),
                                                   batch, _p(g), _p(loss), _s(s)))
        return g, loss

    def train_step(self, x_pool: torch.Tensor, t_pool: torch.Tensor, rows: torch.Tensor | None = None,
                   batch: int | None = None, lr: float = 1e-3, betas=(0.9, 0.999), eps: float = 1e-8,
                   stream=None) -> torch.Tensor:
        """One Adam step; returns the (device) loss before the step."""
        batch = batch or (rows.shape[0] if rows is not None else x_pool.shape[0])
        _lib.check(self.lib.cr_predictor_train_step(self.handle, _p(x_pool), _p(t_pool), x_pool.shape[0], _p(rows),
                                                     batch, lr, betas[0], betas[1], eps, _p(self._loss), _s(stream)))
        return self._loss

    def set_loss_weights(self, weights: np.ndarray | None) -> None:
        """Per-output weights of the squared error (None: equal weights)."""
        if weights is None:
            _lib.check(self.lib.cr_predictor_set_loss_weights(self.handle, None, 0))
            return
        a = np.ascontiguousarray(weights, dtype=np.float32)
        _lib.check(self.lib.cr_predictor_set_loss_weights(self.handle, a.ctypes.data_as(C.POINTER(C.c_float)), a.size))

    def bad_rows(self, reset: bool = True) -> bool:
        """True if a batch named a row outside its pool since the last reset."""
        f = C.c_int32()
        _lib.check(self.lib.cr_predictor_bad_rows(self.handle, C.byref(f), int(reset)))
        return f.value != 0


# ------------------------------------------------------------ queue features
def queue_layout(raster) -> dict:
    """Bin/tile grid of the raster's last draw."""
    lay = _lib.QueueLayout()
    _lib.check(_lib.load().cr_get_queue_layout(raster._ctx, C.byref(lay)), raster._ctx)
    return {k: int(getattr(lay, k)) for k, _ in lay._fields_}


def queue_counts(raster, bins: torch.Tensor | None, tiles: torch.Tensor | None,
                 counters: torch.Tensor | None = None, stream=None) -> None:
    """Copy the last draw's per-bin / per-tile entry counts and its 8 device
    counters into int32 device tensors (ordered on `stream`)."""
    lib = _lib.load()
    _lib.check(lib.cr_queue_counts(raster._ctx, _p(bins), 0 if bins is None else bins.numel(), _p(tiles),
                                   0 if tiles is None else tiles.numel(), _p(counters), _s(stream)), raster._ctx)


def queue_features(bins: torch.Tensor, bins_x: int, bins_y: int, camera_delta, out: torch.Tensor,
                   stream=None) -> torch.Tensor:
    cam = (C.c_float * 6)(*[float(v) for v in camera_delta])
    _lib.check(_lib.load().cr_queue_features(_p(bins), bins_x, bins_y, cam, _p(out), _s(stream)))
    return out


def queue_log_counts(bins, tiles, lay: dict, out: torch.Tensor, stream=None) -> torch.Tensor:
    """out: 2*num_bins + 6 floats (8-byte aligned); see cr_queue_log_counts."""
    _lib.check(_lib.load().cr_queue_log_counts(_p(bins), _p(tiles), lay["bins_x"], lay["bins_y"], lay["tiles_x"],
                                               lay["tiles_y"], lay["bin_log2"], _p(out), _s(stream)))
    return out


def queue_targets(logs_prevprev, logs_prev, logs_cur, out, n_trend: int = 2, stream=None) -> torch.Tensor:
    _lib.check(_lib.load().cr_queue_targets(_p(logs_prevprev), _p(logs_prev), _p(logs_cur), out.numel(), n_trend,
                                            _p(out), _s(stream)))
    return out


def queue_plan(logs_prevprev, logs_prev, prediction, num_bins: int, totals: torch.Tensor, per_bin=None,
               stream=None):
    _lib.check(_lib.load().cr_queue_plan(_p(logs_prevprev), _p(logs_prev), _p(prediction), num_bins, _p(per_bin),
                                         _p(totals), _s(stream)))
    return totals


def predictor_frame(net: Network, bins: int, tiles: int, counters: int | None, layout, ahead: int, logs_prev,
                    logs_cur, logs_target_base, logs_target_trend, target, camera_delta_ahead, x_next, per_bin,
                    fetch, stream=None) -> None:
    """cr_predictor_frame: bins/tiles/counters are device addresses (ints),
    layout a dict or QueueLayout, the rest device tensors (or None)."""
    lay = layout if isinstance(layout, _lib.QueueLayout) else \
        _lib.QueueLayout(**{k: int(layout.get(k, 0)) for k, _ in _lib.QueueLayout._fields_})
    cam = (C.c_float * 6)(*[float(v) for v in camera_delta_ahead])
    _lib.check(_lib.load().cr_predictor_frame(net.handle, bins, tiles, counters, C.byref(lay), int(ahead),
                                              _p(logs_prev), _p(logs_cur), _p(logs_target_base),
                                              _p(logs_target_trend), _p(target), cam, _p(x_next), _p(per_bin),
                                              _p(fetch), _s(stream)))


def queue_buffers(raster):
    """Device pointers (ints) to the raster's last per-bin counts, per-tile
    counts and 8 counters (valid until its next draw)."""
    b, t, c = C.c_void_p(), C.c_void_p(), C.c_void_p()
    _lib.check(_lib.load().cr_get_queue_buffers(raster._ctx, C.byref(b), C.byref(t), C.byref(c)), raster._ctx)
    return b.value, t.value, c.value


class QueuePredictor:
    """Online occupancy predictor for the successive draws of one CudaRaster.

    At frame k the network predicts frame k + ahead: per-bin log ratios of
    the bin- and tile-queue occupancy to frame k's, plus two total heads that
    correct the extrapolated trend of the bin- and tile-entry totals (an
    untrained network, whose output layer starts at zero, predicts that
    trend). ahead = 2 lets a host keep one frame queued while the previous one
    is checked.

    Per frame, after the draw and in stream order: ``step(raster, k,
    camera_delta_ahead)`` -- one fused launch (cr_predictor_frame) that turns
    the draw's counts into frame k's logs, completes the sample of frame
    k - ahead and predicts frame k + ahead -- and one 64-byte copy to the
    host. After a sync the host reads ``predicted_totals(k + ahead)`` and
    ``counters_of(k)``, and sizes that draw with ``capacity()``. ``train``
    takes Adam steps on random mini-batches of the samples whose target
    frames have been checked. Sample k pairs frame k's input (pooled
    histogram and camera move, x_pool[k % pool]) with the change to frame
    k + ahead (t_pool[k % pool]).
    """

    def __init__(self, layout: dict, ahead: int = 1, pool: int = 64, batch: int = 32, lr: float = 3e-4,
                 hidden=(64, 64), seed: int = 0, min_margin: float = 0.005, margin_window: int = 32,
                 margin_factor: float = 1.5):
        self.lay = dict(layout)
        nb, nt = self.lay["num_bins"], self.lay["num_tiles"]
        if self.lay.get("num_instances", 1) != 1:
            raise ValueError("QueuePredictor follows single-instance draws")
        if pool < 2 or ahead < 1:
            raise ValueError("need pool >= 2 and ahead >= 1")
        self.nb, self.nt, self.ahead = nb, nt, ahead
        self.ring = ahead + 2
        self.outputs = 2 * nb + 2
        self.net = Network(HIST_INPUTS, hidden[0], hidden[1], self.outputs, max_batch=max(batch, 1), seed=seed)
        self.layout_c = _lib.QueueLayout(**{k: int(self.lay.get(k, 0)) for k, _ in _lib.QueueLayout._fields_})
        dev = "cuda"
        self.logs = torch.zeros((self.ring, 2 * nb + 6), dtype=torch.float32, device=dev)
        self.x_pool = torch.zeros((pool, HIST_INPUTS), dtype=torch.float32, device=dev)
        self.t_pool = torch.zeros((pool, self.outputs), dtype=torch.float32, device=dev)
        self.per_bin = torch.zeros(2 * nb, dtype=torch.float32, device=dev)
        self.fetch_dev = torch.zeros((self.ring, 8), dtype=torch.float64, device=dev)  # 4 totals, 8 int32 counters
        self.fetch_host = torch.zeros((self.ring, 8), dtype=torch.float64).pin_memory()
        self._host = self.fetch_host.numpy()
        self.gen = torch.Generator(device=dev)
        self.gen.manual_seed(seed)
        self.pool, self.batch, self.lr = pool, batch, lr
        self.stepped = -1       # latest frame stepped
        self.min_margin, self.margin_factor = min_margin, margin_factor
        self.errors = {"bin": deque(maxlen=margin_window), "tile": deque(maxlen=margin_window)}

    # -------------------------------------------------------------- per frame
    def step(self, raster, frame: int, camera_delta_ahead, stream=None) -> None:
        """Frame `frame` was drawn by `raster` (or redrawn: stepping a frame
        again overwrites what it wrote). camera_delta_ahead: the camera move
        from this frame to frame + ahead."""
        k, R, A = frame, self.ring, self.ahead
        bins, tiles, ctrs = queue_buffers(raster)
        lp = self.logs[(k - 1) % R] if k >= 1 else None
        base = self.logs[(k - A) % R] if k >= A else None
        trend = self.logs[(k - A - 1) % R] if k >= A + 1 else None
        target = self.t_pool[(k - A) % self.pool] if k >= A else None
        s = stream or torch.cuda.current_stream()
        predictor_frame(self.net, bins, tiles, ctrs, self.layout_c, A, lp, self.logs[k % R], base, trend, target,
                        camera_delta_ahead, self.x_pool[k % self.pool], self.per_bin, self.fetch_dev[k % R], s)
        with torch.cuda.stream(s):
            self.fetch_host[k % R].copy_(self.fetch_dev[k % R], non_blocking=True)
        self.stepped = max(self.stepped, k)

    def train(self, steps: int, checked_upto: int, stream=None):
        """Adam steps on random mini-batches of the samples whose target frame
        is at most `checked_upto` and whose input is still in the pool."""
        newest = checked_upto - self.ahead
        oldest = max(0, self.stepped - self.pool + 1)
        avail = newest - oldest + 1
        if avail <= 0:
            return None
        b = min(self.batch, avail)
        loss = None
        s = stream or torch.cuda.current_stream()
        with torch.cuda.stream(s):   # the row indices are made, used and freed on the predictor's stream
            for _ in range(steps):
                r = torch.randint(0, avail, (b,), generator=self.gen, device="cuda", dtype=torch.int32)
                rows = torch.remainder(newest - r, self.pool).to(torch.int32)
                loss = self.net.train_step(self.x_pool, self.t_pool, rows, b, lr=self.lr, stream=s)
        return loss

    def predicted_totals(self, frame: int) -> tuple[float, float]:
        """Bin- and tile-entry totals predicted for `frame` (total heads), made
        at frame - ahead."""
        h = self._host[(frame - self.ahead) % self.ring]
        return float(h[0]), float(h[1])

    def per_bin_totals(self, frame: int) -> tuple[float, float]:
        """The same totals summed from the per-bin predictions."""
        h = self._host[(frame - self.ahead) % self.ring]
        return float(h[2]), float(h[3])

    def counters_of(self, frame: int) -> np.ndarray:
        """The 8 device counters of a stepped frame (extra subtriangles, bin
        entries, coarse units, tile entries, fine tiles, overflow flags, and
        the two coarse work counters)."""
        return self._host[frame % self.ring][4:].view(np.int32)

    # ---------------------------------------------------------------- sizing
    def score(self, predicted: tuple[float, float], actual: tuple[float, float]) -> None:
        """Feed the relative error of a prediction into the margin estimate."""
        for k, p, a in (("bin", predicted[0], actual[0]), ("tile", predicted[1], actual[1])):
            self.errors[k].append(a / max(p, 1.0) - 1.0)

    def margin(self, kind: str) -> float:
        e = self.errors[kind]
        worst = max(e) if e else 0.25
        return max(self.min_margin, self.margin_factor * max(worst, 0.0))

    def capacity(self, predicted: tuple[float, float], slack: int = 4096) -> tuple[int, int]:
        """Bin- and tile-entry capacities for the predicted totals."""
        return (int(predicted[0] * (1.0 + self.margin("bin"))) + slack,
                int(predicted[1] * (1.0 + self.margin("tile"))) + slack)

    def close(self) -> None:
        self.net.close()
