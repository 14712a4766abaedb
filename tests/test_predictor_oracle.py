"""CPU checks of the predictor's oracle (no GPU): analytic gradients against
central finite differences, BF16 rounding at the bit level, the Adam step and
the queue-feature arithmetic on hand-made counts."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo


def _rand_params(dims, rng):
    P = mo.layout(*dims)["P"]
    return rng.normal(0.0, 0.5, P)


@pytest.mark.parametrize("dims,batch", [((7, 5, 4, 3), 4), ((20, 8, 8, 6), 5)])
def test_gradients_match_finite_differences(dims, batch):
    rng = np.random.default_rng(1)
    p = _rand_params(dims, rng)
    x = rng.normal(0, 1, (batch, dims[0]))
    t = rng.normal(0, 1, (batch, dims[3]))
    loss, g = mo.loss_and_grad(p, dims, x, t)
    h = 1e-6
    fd = np.empty_like(p)
    for i in range(p.size):
        e = np.zeros_like(p)
        e[i] = h
        fd[i] = (mo.loss_and_grad(p + e, dims, x, t)[0] - mo.loss_and_grad(p - e, dims, x, t)[0]) / (2 * h)
    assert loss > 0
    np.testing.assert_allclose(g, fd, rtol=1e-5, atol=1e-8)


def test_bf16_rounding_bits():
    cases = {0x3F800000: 0x3F80,   # 1.0 exact
             0x3F808000: 0x3F80,   # tie, even stays
             0x3F818000: 0x3F82,   # tie, odd rounds up
             0x3F808001: 0x3F81,   # above the tie
             0x3F807FFF: 0x3F80,   # below the tie
             0xBF818000: 0xBF82,   # sign carried
             0x00000000: 0x0000,
             0x7F7F8000: 0x7F80}   # rounds up to infinity
    src = np.array(list(cases), dtype=np.uint32).view(np.float32)
    got = mo.bf16_bits(src)
    assert [int(v) for v in got] == list(cases.values())


def test_adam_step_first_iteration():
    # With zero moments the first bias-corrected step is lr * g / (|g| + eps).
    g = np.array([0.5, -2.0, 0.0])
    w, m, v = mo.adam_step(np.array([1.0, 1.0, 1.0]), np.zeros(3), np.zeros(3), g, 1, 0.1, 0.9, 0.999, 1e-8)
    np.testing.assert_allclose(w, [1.0 - 0.1 * 0.5 / (0.5 + 1e-8), 1.0 + 0.1 * 2.0 / (2.0 + 1e-8), 1.0])
    np.testing.assert_allclose(m, 0.1 * g)
    np.testing.assert_allclose(v, 0.001 * g * g)


def test_features_pool_bins_into_16x16_cells():
    # 30 x 17 bins (3840x2160 with 128-px bins): cell cx takes bins with bx*16//30 == cx.
    bx, by = 30, 17
    counts = np.arange(bx * by, dtype=np.int64)
    x = mo.features(counts, bx, by, [1, 2, 3, 4, 5, 6])
    lg = np.log1p(counts.reshape(by, bx).astype(np.float64))
    for cy in range(16):
        for cx in range(16):
            sel = [(j, i) for j in range(by) for i in range(bx) if i * 16 // bx == cx and j * 16 // by == cy]
            want = np.mean([lg[j, i] for j, i in sel]) * 0.125 if sel else 0.0
            assert x[cy * 16 + cx] == pytest.approx(want)
    assert list(x[256:]) == [1, 2, 3, 4, 5, 6]
    # Fewer bins than cells: unmapped cells are zero.
    x = mo.features(np.full(4 * 3, 7), 4, 3, [0] * 6)
    assert (x[:256] > 0).sum() == 12


def test_log_counts_targets_and_plan():
    bins_x, bins_y, tiles_x, tiles_y, bl = 2, 2, 3, 3, 1   # 2x2-tile bins, ragged right/bottom
    tiles = np.arange(9)
    bins = np.array([5, 0, 2, 9])
    logs = mo.log_counts(bins, tiles, bins_x, bins_y, tiles_x, tiles_y, bl)
    sums = [0 + 1 + 3 + 4, 2 + 5, 6 + 7, 8]
    np.testing.assert_allclose(logs, np.log1p(np.r_[bins, sums, 16, 36].astype(float)))
    per, tot = mo.plan(None, logs, np.zeros(10), 4)
    np.testing.assert_allclose(per, np.r_[bins, sums])
    np.testing.assert_allclose(tot, [16, 36, 16, 36])
    # Trend: the bin total went 8 -> 16 in the last step, so its head extrapolates to about 32.
    prev = logs.copy()
    prev[-2:] = np.log1p([8.0, 18.0])
    cur = logs.copy()
    cur[-2:] = np.log1p([16.0, 36.0])
    _, tot = mo.plan(prev, cur, np.zeros(10), 4)
    assert tot[0] == pytest.approx(np.expm1(2 * np.log1p(16.0) - np.log1p(8.0)))
    nxt = cur.copy()
    nxt[-2:] = np.log1p([40.0, 80.0])
    t = mo.targets(prev, cur, nxt)
    np.testing.assert_allclose(t[:-2], 0.0, atol=1e-12)
    np.testing.assert_allclose(t[-2:], (nxt - cur)[-2:] - (cur - prev)[-2:])
