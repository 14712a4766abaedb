"""CPU oracle of the learned queue predictor -- test infrastructure only.

Restates, in float64 numpy, the network and the queue-feature arithmetic that
cudaraster-linux_gb300/csrc/predictor.cu runs on the GPU, so that the GPU's
forward pass, gradients, Adam step and feature kernels can be checked against
it. The reference has no learned part (it sizes queues from the previous draw
and grows them on overflow, src/cudaraster/CudaRaster.cpp:263-275, 325-342);
this oracle is pinned instead by central finite differences of its own loss
(tests/test_predictor_oracle.py), and BF16 rounding by bit-level cases.

Network: x[inputs] -> GELU(W1 x + b1) -> GELU(W2 . + b2) -> W3 . + b3, with
the parameters rounded to BF16 before use; loss = the squared error averaged
over the batch and, with per-output weights, over the outputs. Flat parameter layout: W1[h1][in], b1, W2[h2][h1], b2,
W3[out][h2], b3.
"""
from __future__ import annotations

import math

import numpy as np

try:
    from scipy.special import erf as _erf
except ImportError:  # pragma: no cover - scipy is present on both machines
    _erf = np.vectorize(math.erf)

HIST_CELLS = 16
HIST_SCALE = 0.125


def bf16_round(x: np.ndarray) -> np.ndarray:
    """float32 -> nearest-even BF16, returned as float32 (finite inputs)."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF
    return (r.astype(np.uint32) << 16).view(np.float32)


def bf16_bits(x: np.ndarray) -> np.ndarray:
    return (bf16_round(x).view(np.uint32) >> 16).astype(np.uint16)


def layout(inputs: int, h1: int, h2: int, outputs: int) -> dict:
    o = {}
    o["W1"] = 0
    o["b1"] = o["W1"] + h1 * inputs
    o["W2"] = o["b1"] + h1
    o["b2"] = o["W2"] + h2 * h1
    o["W3"] = o["b2"] + h2
    o["b3"] = o["W3"] + outputs * h2
    o["P"] = o["b3"] + outputs
    return o


def unpack(params: np.ndarray, dims) -> dict:
    inputs, h1, h2, outputs = dims
    o = layout(*dims)
    p = np.asarray(params, dtype=np.float64)
    return {"W1": p[o["W1"]:o["b1"]].reshape(h1, inputs), "b1": p[o["b1"]:o["W2"]],
            "W2": p[o["W2"]:o["b2"]].reshape(h2, h1), "b2": p[o["b2"]:o["W3"]],
            "W3": p[o["W3"]:o["b3"]].reshape(outputs, h2), "b3": p[o["b3"]:o["P"]]}


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def forward(params: np.ndarray, dims, x: np.ndarray) -> dict:
    """params: the values the network uses (already BF16-rounded); float64 math."""
    w = unpack(params, dims)
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ w["W1"].T + w["b1"]
    a1 = gelu(z1)
    z2 = a1 @ w["W2"].T + w["b2"]
    a2 = gelu(z2)
    y = a2 @ w["W3"].T + w["b3"]
    return {"x": x, "z1": z1, "a1": a1, "z2": z2, "a2": a2, "y": y}


def loss_and_grad(params: np.ndarray, dims, x: np.ndarray, t: np.ndarray, weights=None):
    """Weighted mean squared error: sum(w_o (y - t)^2) / (batch * sum(w_o)),
    w = 1 when weights is None; returns (loss, flat gradient)."""
    w = unpack(params, dims)
    f = forward(params, dims, x)
    t = np.asarray(t, dtype=np.float64)
    wo = np.ones(dims[3]) if weights is None else np.asarray(weights, np.float64)
    n = f["y"].shape[0] * wo.sum()
    e = f["y"] - t
    loss = float((wo * e * e).sum() / n)
    dy = 2.0 * wo * e / n
    g = {}
    g["W3"] = dy.T @ f["a2"]
    g["b3"] = dy.sum(0)
    dz2 = (dy @ w["W3"]) * gelu_grad(f["z2"])
    g["W2"] = dz2.T @ f["a1"]
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ w["W2"]) * gelu_grad(f["z1"])
    g["W1"] = dz1.T @ f["x"]
    g["b1"] = dz1.sum(0)
    flat = np.concatenate([g[k].reshape(-1) for k in ("W1", "b1", "W2", "b2", "W3", "b3")])
    return loss, flat


def adam_step(master, m, v, g, step: int, lr: float, b1: float, b2: float, eps: float):
    """Bias-corrected Adam in float64; returns new (master, m, v)."""
    master = np.asarray(master, np.float64)
    m = b1 * np.asarray(m, np.float64) + (1.0 - b1) * g
    v = b2 * np.asarray(v, np.float64) + (1.0 - b2) * g * g
    c1 = 1.0 - b1 ** step
    c2 = 1.0 - b2 ** step
    return master - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v


# ------------------------------------------------------------------ features
def features(bin_counts: np.ndarray, bins_x: int, bins_y: int, camera_delta) -> np.ndarray:
    c = np.asarray(bin_counts, np.float64).reshape(bins_y, bins_x)
    lg = np.log1p(c)
    x = np.zeros(HIST_CELLS * HIST_CELLS + 6)
    for cy in range(HIST_CELLS):
        by0, by1 = -(-cy * bins_y // HIST_CELLS), -(-(cy + 1) * bins_y // HIST_CELLS)
        for cx in range(HIST_CELLS):
            bx0, bx1 = -(-cx * bins_x // HIST_CELLS), -(-(cx + 1) * bins_x // HIST_CELLS)
            blk = lg[by0:by1, bx0:bx1]
            x[cy * HIST_CELLS + cx] = blk.mean() * HIST_SCALE if blk.size else 0.0
    x[HIST_CELLS * HIST_CELLS:] = np.asarray(camera_delta, np.float64)
    return x


def log_counts(bin_counts, tile_counts, bins_x, bins_y, tiles_x, tiles_y, bin_log2) -> np.ndarray:
    """[log1p(bin entries) per bin, log1p(tile entries of the bin's tiles) per
    bin, log1p(total bin entries), log1p(total tile entries)]."""
    side = 1 << bin_log2
    t = np.asarray(tile_counts, np.int64).reshape(tiles_y, tiles_x)
    pad = np.zeros((bins_y * side, bins_x * side), np.int64)
    pad[:tiles_y, :tiles_x] = t
    sums = pad.reshape(bins_y, side, bins_x, side).sum(axis=(1, 3)).reshape(-1)
    b = np.asarray(bin_counts, np.int64)
    return np.concatenate([np.log1p(b.astype(np.float64)), np.log1p(sums.astype(np.float64)),
                           np.log1p([float(b.sum()), float(sums.sum())])])


def targets(logs_prevprev, logs_prev, logs_cur, n_trend: int = 2) -> np.ndarray:
    """cur - prev; the last n_trend entries also lose the previous step's trend."""
    t = np.asarray(logs_cur, np.float64) - np.asarray(logs_prev, np.float64)
    if logs_prevprev is not None and n_trend:
        t[-n_trend:] -= (np.asarray(logs_prev, np.float64) - np.asarray(logs_prevprev, np.float64))[-n_trend:]
    return t


def plan(logs_prevprev, logs_prev, prediction, num_bins: int):
    """Per-bin occupancy (2nb values) and totals [bin head, tile head, sum of
    per-bin bin predictions, sum of per-bin tile predictions]."""
    lp = np.asarray(logs_prev, np.float64)
    y = np.asarray(prediction, np.float64)
    n2 = 2 * num_bins
    per = np.maximum(np.expm1(lp[:n2] + y[:n2]), 0.0)
    base = lp[n2:n2 + 2].copy()
    if logs_prevprev is not None:
        base += lp[n2:n2 + 2] - np.asarray(logs_prevprev, np.float64)[n2:n2 + 2]
    heads = np.maximum(np.expm1(base + y[n2:n2 + 2]), 0.0)
    return per, np.array([heads[0], heads[1], per[:num_bins].sum(), per[num_bins:].sum()])
