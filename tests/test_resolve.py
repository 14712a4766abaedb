"""MSAA resolve (cr_resolve_color) against a numpy restatement of its rule,
and the PPM writer."""
import numpy as np
import pytest
import torch

from conftest import pkg_mod
from helpers import PIPE_SAMPLES, gpu_render, pkg


def resolve_reference(words: np.ndarray, width: int, height: int, samples: int) -> np.ndarray:
    """Per channel (sum of the pixel's samples + S/2) >> log2 S, from the
    surface layout (sample i of pixel x at word (x >> 3) * 8 * S + i * 8 + (x & 7))."""
    w = words.reshape(words.shape[0], -1)[:height]
    log2 = samples.bit_length() - 1
    x = np.arange(width)
    cols = (x >> 3) * 8 * samples + (x & 7)
    acc = np.zeros((height, width, 4), np.uint32)
    for i in range(samples):
        v = w[:, cols + i * 8].astype(np.uint32)
        for k in range(4):
            acc[..., k] += (v >> (8 * k)) & 0xFF
    return ((acc + (samples >> 1)) >> log2).astype(np.uint8)


def test_ppm_writer(tmp_path):
    img = np.arange(2 * 3 * 4, dtype=np.uint8).reshape(2, 3, 4)
    pkg().write_ppm(tmp_path / "a.ppm", img)
    data = (tmp_path / "a.ppm").read_bytes()
    assert data.startswith(b"P6\n3 2\n255\n")
    assert data[len(b"P6\n3 2\n255\n"):] == img[..., :3].tobytes()


def test_reference_rule_on_known_values():
    # Two samples of one pixel: channels (10, 20, 30, 255) and (11, 21, 30, 0) -> rounded half up.
    a = np.uint32(10 | 20 << 8 | 30 << 16 | 255 << 24)
    b = np.uint32(11 | 21 << 8 | 30 << 16 | 0 << 24)
    words = np.zeros((8, 16), np.uint32)
    words[0, 0], words[0, 8] = a, b
    out = resolve_reference(words, 1, 1, 2)
    assert list(out[0, 0]) == [11, 21, 30, 128]


@pytest.mark.gpu
@pytest.mark.parametrize("pipe", ["PixelPipe_gouraud", "PixelPipe_gouraud_msaa2", "PixelPipe_gouraud_srcover_msaa4",
                                  "PixelPipe_gouraud_msaa8"])
def test_resolve_matches_rule(cuda, pipe):
    p = pkg()
    sc = pkg_mod("scenes").soup(20000, 333, 250, seed=41, median_px=6.0,
                                alpha_range=(0.2, 1.0) if "srcover" in pipe else None)
    s = PIPE_SAMPLES.get(pipe, 1)
    clear = (p.color_to_abgr(0.1, 0.2, 0.3, 1.0), p.clear_depth_from_float(1.0))
    gc, _, _, _ = gpu_render(pipe, sc, clear)
    surf = p.CudaSurface((333, 250), p.CudaSurface.FORMAT_RGBA8, s)
    surf.tensor.copy_(torch.from_numpy(gc.view(np.int32)))
    got = surf.resolve().cpu().numpy()
    want = resolve_reference(gc, 333, 250, s)
    assert got.shape == (250, 333, 4)
    np.testing.assert_array_equal(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("samples", [1, 2, 4, 8])
def test_resolve_random_words(cuda, samples):
    # Every byte value in every sample, including all-255 pixels (the largest lane sums).
    p = pkg()
    w, h = 203, 77
    surf = p.CudaSurface((w, h), p.CudaSurface.FORMAT_RGBA8, samples)
    rng = np.random.default_rng(samples)
    words = rng.integers(0, 2**32, tuple(surf.tensor.shape), dtype=np.uint64).astype(np.uint32)
    words[::5] = 0xFFFFFFFF
    surf.tensor.copy_(torch.from_numpy(words.view(np.int32)))
    got = surf.resolve().cpu().numpy()
    np.testing.assert_array_equal(got, resolve_reference(words, w, h, samples))
