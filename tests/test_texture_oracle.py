"""Known answers of the oracle's atlas filter and of the exactly specified
shader arithmetic, and agreement between its C++ and numpy restatements."""
import numpy as np

from oracle import oracle as orc
from oracle import vertex_oracle as vo


def _atlas(seed=0, h=4, w=8):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 2**32, (h, w), dtype=np.uint64).astype(np.uint32)


def _channels(word):
    return np.array([(int(word) >> (8 * k)) & 255 for k in range(4)], np.float64)


def test_texel_centres_return_texels():
    a = _atlas()
    h, w = a.shape
    uv = np.array([[(x + 0.5) / w, (y + 0.5) / h] for y in range(h) for x in range(w)], np.float32)
    out = orc.texture_sample(a, uv)
    want = np.array([_channels(a[y, x]) / 255.0 for y in range(h) for x in range(w)], np.float32)
    assert np.array_equal(out, want)


def test_half_way_points_average():
    a = _atlas(1)
    h, w = a.shape
    out = orc.texture_sample(a, np.array([[1.0 / w, 0.5 / h]], np.float32))[0]
    want = (_channels(a[0, 0]) + _channels(a[0, 1])) * 128 * 256 / 16711680.0
    assert np.allclose(out, want.astype(np.float32), atol=0, rtol=1e-7)


def test_wrap_addressing():
    a = _atlas(2)
    h, w = a.shape
    # u = 0 sits half-way between the last and the first column; whole-number shifts wrap.
    base = orc.texture_sample(a, np.array([[0.0, 0.5 / h]], np.float32))[0]
    want = (_channels(a[0, w - 1]) + _channels(a[0, 0])) * 128 * 256 / 16711680.0
    assert np.allclose(base, want.astype(np.float32), atol=0, rtol=1e-7)
    for shift in (-3.0, -1.0, 1.0, 5.0):
        uv = np.array([[0.3 + shift, 0.6 - shift]], np.float32)
        assert np.array_equal(orc.texture_sample(a, uv), orc.texture_sample(a, np.array([[0.3, 0.6]], np.float32)))


def test_weights_are_eight_bit():
    # Offsets closer than 1/512 of a texel round to the same weight.
    a = _atlas(3)
    h, w = a.shape
    x = (2.0 + 0.5 + 0.25) / w
    uv = np.array([[x, 0.5 / h], [x + 0.5 / 1024 / w, 0.5 / h]], np.float32)
    out = orc.texture_sample(a, uv)
    assert np.array_equal(out[0], out[1])


def test_non_finite_coordinates_are_defined():
    a = _atlas(4)
    uv = np.array([[np.nan, 0.5], [np.inf, -np.inf], [0.0, 0.0]], np.float32)
    out = orc.texture_sample(a, uv)
    assert np.all(np.isfinite(out))
    assert np.array_equal(out[1], out[2])   # non-finite coordinates read as 0


def test_cpp_and_numpy_pow_agree():
    rng = np.random.default_rng(5)
    x = np.concatenate([rng.uniform(0, 1, 3000), rng.uniform(0, 8, 1000), [0.0, 1e-45, 1e-38, np.inf]]).astype(np.float32)
    y = np.concatenate([rng.uniform(0.25, 128, 3000), rng.uniform(-4, 4, 1000), [2, 3, 0.5, 2]]).astype(np.float32)
    a = vo.pow_exact(x, y)
    b = np.array([orc.pow_exact(float(p), float(q)) for p, q in zip(x, y)], np.float32)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_log2_exact_special_values():
    assert orc.log2_exact(0.0) == -np.inf
    assert np.isnan(orc.log2_exact(-1.0))
    assert orc.log2_exact(np.inf) == np.inf
    for e in range(-149, 128, 7):
        assert orc.log2_exact(float(np.ldexp(np.float32(1), e))) == e


def test_cpp_lighting_matches_vertex_oracle():
    # The fragment shader's evaluateLighting equals the vertex oracle's, vertex by vertex.
    rng = np.random.default_rng(6)
    n = 500
    v = np.zeros((n, 8), np.float32)
    v[:, 0:3] = rng.uniform(-2, 2, (n, 3))
    v[:, 3:6] = rng.normal(size=(n, 3))
    mats = np.zeros((1, 8), np.float32)
    mats[0] = [0.6, 0.5, 0.4, 1.0, 0.3, 0.3, 0.3, 17.0]
    eye = np.eye(4, dtype=np.float32)
    out = vo.vertex_gouraud(v, eye, eye, eye[:3, :3].copy(), mats, np.zeros(n, np.int32))
    for i in range(n):
        c = orc.evaluate_lighting(v[i, 0:3], v[i, 3:6], mats[0, 4:7], mats[0, 7], mats[0, 0:3])
        assert np.array_equal(c.view(np.uint32), out[i, 4:7].view(np.uint32))


def test_division_free_normalisation_is_exact():
    # The GPU filter divides its weighted sums by 255 * 65536 with a multiplication and
    # two FMAs; over every sum it can form that equals the IEEE division bit for bit.
    assert orc.load().or_tex_normalize_mismatches() == 0
