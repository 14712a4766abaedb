"""The learned queue predictor's kernels against the float64 oracle: forward
pass, gradients of every parameter tensor, Adam steps, the BF16 parameter
copy, the queue-feature kernels, and the counts a draw exports."""
import numpy as np
import pytest
import torch

from conftest import pkg_mod
from helpers import pkg
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu

DIMS = (262, 64, 64, 1020)   # 16x16 histogram + 6 camera floats -> 2 x 510 bins (3840x2160, 128-px bins)
NAMES = ("W1", "b1", "W2", "b2", "W3", "b3")


def _net(seed=0, noise=0.05, dims=DIMS):
    P = pkg_mod("predictor")
    net = P.Network(*dims, max_batch=64, seed=seed)
    rng = np.random.default_rng(seed + 10)
    net.set_params(net.get_params() + rng.normal(0.0, noise, net.num_params).astype(np.float32))
    return net


def _pools(rng, n=40):
    x = rng.normal(0.0, 1.0, (n, DIMS[0])).astype(np.float32)
    t = rng.normal(0.0, 0.5, (n, DIMS[3])).astype(np.float32)
    return x, t, torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()


def _check_grads(g, ref, tol=2e-4):
    lay = mo.layout(*DIMS)
    bounds = [lay[k] for k in NAMES] + [lay["P"]]
    for i, name in enumerate(NAMES):
        a, b = g[bounds[i]:bounds[i + 1]], ref[bounds[i]:bounds[i + 1]]
        scale = np.abs(b).max()
        assert scale > 0, name
        err = np.abs(a - b).max() / scale
        assert err < tol, f"{name}: relative error {err:.2e}"


def test_bf16_copy_is_rounded_master(cuda):
    net = _net()
    assert np.array_equal(net.get_params_bf16().view(np.uint32), mo.bf16_round(net.get_params()).view(np.uint32))


def test_forward_matches_oracle(cuda):
    net = _net()
    rng = np.random.default_rng(1)
    x = rng.normal(0.0, 1.0, (16, DIMS[0])).astype(np.float32)
    y = net.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    ref = mo.forward(net.get_params_bf16(), DIMS, x)["y"]
    assert np.abs(y - ref).max() / np.abs(ref).max() < 2e-5


def test_gradients_match_oracle(cuda):
    net = _net(seed=3)
    rng = np.random.default_rng(2)
    x, t, xd, td = _pools(rng)
    rows = np.array([3, 17, 5, 39, 0, 22, 8, 8, 31, 12], dtype=np.int32)   # repeats allowed
    g, loss = net.gradients(xd, td, torch.from_numpy(rows).cuda())
    ref_loss, ref_g = mo.loss_and_grad(net.get_params_bf16(), DIMS, x[rows], t[rows])
    assert float(loss.item()) == pytest.approx(ref_loss, rel=2e-5)
    _check_grads(g.cpu().numpy(), ref_g)


def test_adam_steps_match_oracle(cuda):
    net = _net(seed=4)
    rng = np.random.default_rng(5)
    x, t, xd, td = _pools(rng)
    rows = torch.from_numpy(np.arange(0, 40, 2, dtype=np.int32)).cuda()
    lr, b1, b2, eps = 1e-3, 0.9, 0.999, 1e-8
    master = net.get_params().astype(np.float64)
    m = np.zeros_like(master)
    v = np.zeros_like(master)
    for step in (1, 2, 3):
        g, _ = net.gradients(xd, td, rows)
        net.train_step(xd, td, rows, lr=lr, betas=(b1, b2), eps=eps)
        master, m, v = mo.adam_step(master, m, v, g.cpu().numpy().astype(np.float64), step, lr, b1, b2, eps)
        got = net.get_params()
        np.testing.assert_allclose(got, master, rtol=0, atol=2e-6)
        master = got.astype(np.float64)    # follow the device's FP32 rounding
        assert np.array_equal(net.get_params_bf16().view(np.uint32), mo.bf16_round(got).view(np.uint32))
    assert net.steps == 3


def test_training_fits_a_teacher(cuda):
    P = pkg_mod("predictor")
    rng = np.random.default_rng(7)
    teacher = P.init_params(DIMS, seed=11)
    lay = mo.layout(*DIMS)
    teacher[lay["W3"]:lay["P"]] = rng.normal(0.0, 0.2, lay["P"] - lay["W3"])
    x = rng.normal(0.0, 1.0, (64, DIMS[0])).astype(np.float32)
    t = mo.forward(mo.bf16_round(teacher), DIMS, x)["y"].astype(np.float32)
    net = P.Network(*DIMS, max_batch=32, seed=1)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    first = float(net.gradients(xd, td, None, 32)[1].item())
    gen = torch.Generator(device="cuda")
    gen.manual_seed(0)
    for _ in range(400):
        rows = torch.randint(0, 64, (32,), generator=gen, device="cuda", dtype=torch.int32)
        net.train_step(xd, td, rows, lr=3e-3)
    last = float(net.gradients(xd, td, None, 32)[1].item())
    assert last < 0.3 * first, (first, last)


def test_queue_feature_kernels_match_oracle(cuda):
    P = pkg_mod("predictor")
    rng = np.random.default_rng(9)
    lay = {"bins_x": 30, "bins_y": 17, "tiles_x": 480, "tiles_y": 270, "bin_log2": 4}
    nb = 30 * 17
    frames = []
    b = rng.integers(0, 200000, nb)
    t = rng.integers(0, 3000, 480 * 270)
    for k in range(3):
        bk = (b * rng.uniform(0.5, 1.5, nb)).astype(np.int32)
        tk = (t * rng.uniform(0.5, 1.5, t.size)).astype(np.int32)
        bk[k::7] = 0
        tk[k::11] = 0
        frames.append((bk, tk))
    logs, refs = [], []
    for bk, tk in frames:
        out = torch.zeros(2 * nb + 6, device="cuda")
        P.queue_log_counts(torch.from_numpy(bk).cuda(), torch.from_numpy(tk).cuda(), lay, out)
        logs.append(out)
        refs.append(mo.log_counts(bk, tk, 30, 17, 480, 270, 4))
        np.testing.assert_allclose(out[:2 * nb + 2].cpu().numpy(), refs[-1], rtol=2e-6, atol=1e-7)
    cam = [0.5, -0.25, 0.125, 1.0, 0.0, -2.0]
    x = P.queue_features(torch.from_numpy(frames[0][0]).cuda(), 30, 17, cam, torch.empty(262, device="cuda"))
    np.testing.assert_allclose(x.cpu().numpy(), mo.features(frames[0][0], 30, 17, cam), rtol=2e-6, atol=1e-7)
    n = 2 * nb + 2
    for pp in (None, logs[0]):
        tgt = P.queue_targets(pp, logs[1], logs[2], torch.empty(n, device="cuda")).cpu().numpy()
        ref = mo.targets(None if pp is None else refs[0], refs[1], refs[2])
        np.testing.assert_allclose(tgt, ref, rtol=0, atol=1e-5)
        y = torch.from_numpy(rng.normal(0, 0.1, n).astype(np.float32)).cuda()
        per = torch.empty(2 * nb, device="cuda")
        totals = P.queue_plan(pp, logs[2], y, nb, torch.empty(4, dtype=torch.float64, device="cuda"), per)
        ref_per, ref_tot = mo.plan(None if pp is None else logs[0].cpu().numpy(), logs[2].cpu().numpy()[:n],
                                   y.cpu().numpy(), nb)
        np.testing.assert_allclose(per.cpu().numpy(), ref_per, rtol=1e-5, atol=1e-3)
        np.testing.assert_allclose(totals.cpu().numpy(), ref_tot, rtol=1e-5)


def test_queue_counts_of_a_draw(cuda):
    P = pkg_mod("predictor")
    p = pkg()
    sc = pkg_mod("scenes").soup(50000, 640, 480, seed=8, median_px=9.0)
    cr = p.CudaRaster()
    cr.init()
    cs = p.CudaSurface((640, 480), p.CudaSurface.FORMAT_RGBA8, 1)
    ds = p.CudaSurface((640, 480), p.CudaSurface.FORMAT_DEPTH32, 1)
    v = torch.from_numpy(sc["vertices"]).cuda()
    i = torch.from_numpy(sc["indices"]).cuda()
    cr.setSurfaces(cs, ds)
    cr.setPixelPipe(None, "PixelPipe_gouraud")
    cr.setVertexBuffer(v, 0)
    cr.setIndexBuffer(i, 0, i.shape[0])
    cr.deferredClear((0, 0, 0, 1), 1.0)
    cr.drawTriangles()
    lay = P.queue_layout(cr)
    assert (lay["tiles_x"], lay["tiles_y"], lay["num_instances"]) == (80, 60, 1)
    assert lay["num_bins"] == lay["bins_x"] * lay["bins_y"] and lay["num_tiles"] == 80 * 60
    bins = torch.zeros(lay["num_bins"], dtype=torch.int32, device="cuda")
    tiles = torch.zeros(lay["num_tiles"], dtype=torch.int32, device="cuda")
    ctr = torch.zeros(8, dtype=torch.int32, device="cuda")
    P.queue_counts(cr, bins, tiles, ctr)
    c = cr.getCounters()
    assert int(bins.sum()) == c["bin_entries"] > 0
    assert int(tiles.sum()) == c["tile_entries"] > 0
    assert int(ctr[1]) == c["bin_entries"] and int(ctr[3]) == c["tile_entries"] and int(ctr[5]) == 0
    with pytest.raises(p.RasterError):
        P.queue_counts(cr, bins[:-1], tiles)


def test_rows_outside_the_pool_are_flagged_not_read(cuda):
    net = _net(seed=6)
    rng = np.random.default_rng(12)
    x, t, xd, td = _pools(rng, n=40)
    assert not net.bad_rows()
    bad = torch.tensor([3, 40, -1, 1 << 30], dtype=torch.int32, device="cuda")
    g_bad, _ = net.gradients(xd, td, bad)
    assert net.bad_rows()              # flagged, then reset
    assert not net.bad_rows()
    g_ref, _ = net.gradients(xd, td, torch.tensor([3, 0, 0, 0], dtype=torch.int32, device="cuda"))
    assert torch.equal(g_bad, g_ref)
    assert not net.bad_rows()


def test_fused_frame_step_matches_the_separate_kernels_and_oracle(cuda):
    P = pkg_mod("predictor")
    rng = np.random.default_rng(21)
    lay = {"bins_x": 30, "bins_y": 17, "tiles_x": 480, "tiles_y": 270, "bin_log2": 4, "num_bins": 510,
           "num_tiles": 480 * 270, "num_instances": 1}
    nb = 510
    net = _net(seed=8, noise=0.02, dims=(262, 64, 64, 2 * 510 + 2))
    logs = []
    for k in range(2):
        b = rng.integers(0, 100000, nb).astype(np.int32)
        t = rng.integers(0, 2000, 480 * 270).astype(np.int32)
        out = torch.zeros(2 * nb + 6, device="cuda")
        P.queue_log_counts(torch.from_numpy(b).cuda(), torch.from_numpy(t).cuda(), lay, out)
        logs.append(out)
    b = torch.from_numpy(rng.integers(0, 100000, nb).astype(np.int32)).cuda()
    t = torch.from_numpy(rng.integers(0, 2000, 480 * 270).astype(np.int32)).cuda()
    ctr = torch.arange(8, dtype=torch.int32, device="cuda") * 7
    cam = [0.3, 0.0, -0.2, 0.5, 0.1, -0.4]
    cur = torch.zeros(2 * nb + 6, device="cuda")
    target = torch.zeros(2 * nb + 2, device="cuda")
    x = torch.zeros(262, device="cuda")
    per = torch.zeros(2 * nb, device="cuda")
    fetch = torch.zeros(8, dtype=torch.float64, device="cuda")
    P.predictor_frame(net, b.data_ptr(), t.data_ptr(), ctr.data_ptr(), lay, 1, logs[1], cur, logs[1], logs[0],
                      target, cam, x, per, fetch)
    ref_cur = P.queue_log_counts(b, t, lay, torch.zeros(2 * nb + 6, device="cuda"))
    n = 2 * nb + 2
    assert torch.equal(cur[:n], ref_cur[:n])
    assert torch.equal(target, P.queue_targets(logs[0], logs[1], cur, torch.zeros(n, device="cuda")))
    assert torch.equal(x, P.queue_features(b, 30, 17, cam, torch.zeros(262, device="cuda")))
    y = mo.forward(net.get_params_bf16(), DIMS[:3] + (n,), x.cpu().numpy()[None])["y"][0]
    ref_per, ref_tot = mo.plan(logs[1].cpu().numpy()[:n], cur.cpu().numpy()[:n], y, nb)
    np.testing.assert_allclose(per.cpu().numpy(), ref_per, rtol=2e-4, atol=1e-3)
    host = fetch.cpu().numpy()
    np.testing.assert_allclose(host[:4], ref_tot, rtol=2e-4)
    assert list(host[4:].view(np.int32)) == [0, 7, 14, 21, 28, 35, 42, 49]

    # Two frames ahead: the target spans two frames and the heads double the trend.
    target2 = torch.zeros(n, device="cuda")
    P.predictor_frame(net, b.data_ptr(), t.data_ptr(), ctr.data_ptr(), lay, 2, logs[1], cur, logs[1], logs[0],
                      target2, cam, x, per, fetch)
    want = (cur - logs[1])[:n].clone()
    want[-2:] -= 2.0 * (logs[1] - logs[0])[n - 2:n]
    assert torch.allclose(target2, want, rtol=0, atol=1e-6)
    c, pv = cur.cpu().numpy().astype(np.float64)[:n], logs[1].cpu().numpy().astype(np.float64)[:n]
    heads = np.expm1(c[-2:] + 2.0 * (c[-2:] - pv[-2:]) + y[-2:])
    np.testing.assert_allclose(fetch.cpu().numpy()[:2], heads, rtol=2e-4)


def test_weighted_loss_gradients_match_oracle(cuda):
    """Per-output loss weights (cr_predictor_set_loss_weights): loss and every
    gradient against the oracle's weighted squared error; equal weights give
    the unweighted loss back."""
    net = _net(seed=13)
    rng = np.random.default_rng(14)
    x, t, xd, td = _pools(rng)
    rows = np.array([1, 9, 33, 4, 4, 20], dtype=np.int32)
    w = rng.uniform(0.0, 2.0, DIMS[3]).astype(np.float32)
    w[-2:] = 50.0
    net.set_loss_weights(w)
    g, loss = net.gradients(xd, td, torch.from_numpy(rows).cuda())
    ref_loss, ref_g = mo.loss_and_grad(net.get_params_bf16(), DIMS, x[rows], t[rows], weights=w)
    assert float(loss.item()) == pytest.approx(ref_loss, rel=2e-5)
    _check_grads(g.cpu().numpy(), ref_g)
    net.set_loss_weights(None)
    g2, loss2 = net.gradients(xd, td, torch.from_numpy(rows).cuda())
    ref_loss2, ref_g2 = mo.loss_and_grad(net.get_params_bf16(), DIMS, x[rows], t[rows])
    assert float(loss2.item()) == pytest.approx(ref_loss2, rel=2e-5)
    _check_grads(g2.cpu().numpy(), ref_g2)


def test_fused_training_step_time(cuda):
    """One training step (gather, forward, loss, backward, Adam) of the queue
    predictor's network at batch 32 is four launches and under 50 us."""
    net = _net(seed=15, dims=(262, 64, 64, 1022))
    rng = np.random.default_rng(16)
    x = torch.from_numpy(rng.normal(0, 1, (64, 262)).astype(np.float32)).cuda()
    t = torch.from_numpy(rng.normal(0, 0.5, (64, 1022)).astype(np.float32)).cuda()
    rows = torch.arange(32, dtype=torch.int32, device="cuda")
    for _ in range(5):
        net.train_step(x, t, rows, 32)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = 50
    a.record()
    for _ in range(n):
        net.train_step(x, t, rows, 32)
    b.record()
    torch.cuda.synchronize()
    us = a.elapsed_time(b) * 1e3 / n
    print(f"fused training step: {us:.1f} us")
    assert us < 50.0, us
