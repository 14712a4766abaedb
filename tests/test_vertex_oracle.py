"""The vertex shaders' oracle on its own (CPU): its exact power against
float64 pow, its special cases, and the lighting's shape."""
import math

import numpy as np

from oracle import vertex_oracle as vo


def test_pow_exact_close_to_pow():
    rng = np.random.default_rng(3)
    x = rng.uniform(0.0, 1.0, 200_000).astype(np.float32)
    y = rng.uniform(0.25, 128.0, 200_000).astype(np.float32)
    got = vo.pow_exact(x, y).astype(np.float64)
    ref = np.power(x.astype(np.float64), y.astype(np.float64))
    m = ref > 1e-30
    assert np.max(np.abs(got[m] - ref[m]) / ref[m]) < 2e-5


def test_pow_exact_special_cases():
    x = np.array([0.0, 0.0, 0.0, 2.0, np.inf, np.inf, 1e-45, 1.0], np.float32)
    y = np.array([2.0, 0.0, -1.0, 0.0, 3.0, -3.0, 1.0, 7.5], np.float32)
    got = vo.pow_exact(x, y)
    assert got[0] == 0.0 and got[1] == 1.0 and np.isinf(got[2]) and got[3] == 1.0
    assert np.isinf(got[4]) and got[5] == 0.0
    assert abs(float(got[6]) - 1.4e-45) < 1e-45
    assert abs(float(got[7]) - 1.0) < 1e-6


def test_log2_exact_on_powers_of_two_and_subnormals():
    e = np.arange(-149, 128)
    x = np.ldexp(np.ones(e.shape), e).astype(np.float32)
    got = vo.log2_exact(x)
    assert np.all(np.abs(got - e) <= 1e-5 * np.maximum(1, np.abs(e)))
    assert np.all(np.isfinite(vo.exp2_exact(np.linspace(-160, 140, 1001, dtype=np.float32))) |
                  (np.linspace(-160, 140, 1001) >= 128))


def test_gouraud_lighting_shape():
    # Camera at the origin looking down -z at a vertex facing it: full diffuse.
    eye = np.eye(4, dtype=np.float32)
    v = np.array([[0, 0, -5, 0, 0, 1, 0.5, 0.5], [0, 0, -5, 0, 0, -1, 0, 0], [1, 2, 3, 0, 0, 0, 0, 0]], np.float32)
    mats = np.array([[0.8, 0.4, 0.2, 0.9, 0.5, 0.5, 0.5, 16.0]], np.float32)
    out = vo.vertex_gouraud(v, eye, eye, np.eye(3, dtype=np.float32), mats, np.zeros(3, np.int32))
    # Facing: diffuse (1 * 0.75 + 0.25) * colour + specular 1^16 * 0.5.
    assert np.allclose(out[0, 4:7], mats[0, 0:3] + 0.5, atol=1e-6) and out[0, 7] == np.float32(0.9)
    # Facing away: diffuse at its floor 0.25; the reflection of the view ray
    # points back along it, so the reference's specular term is 1^16.
    assert np.allclose(out[1, 4:7], mats[0, 0:3] * 0.25 + 0.5, atol=1e-6)
    # A zero normal normalizes to zero (rcp(0) = 0): no NaN, diffuse floor only.
    assert np.all(np.isfinite(out[2])) and np.allclose(out[2, 4:7], mats[0, 0:3] * 0.25, atol=1e-6)
    assert np.allclose(out[:, 0:4], np.concatenate([v[:, 0:3], np.ones((3, 1))], axis=1))


def test_tex_phong_records():
    rng = np.random.default_rng(4)
    v = rng.normal(size=(50, 8)).astype(np.float32)
    m = rng.normal(size=(4, 4)).astype(np.float32)
    out = vo.vertex_tex_phong(v, m, np.eye(4), np.eye(3))
    assert out.shape == (50, 16)
    assert np.array_equal(out[:, 8:11], v[:, 3:6]) and np.all(out[:, 11] == 0) and np.all(out[:, 15] == 1)
    assert np.array_equal(out[:, 12:14], v[:, 6:8]) and np.all(out[:, 14] == 0)
    assert math.isclose(float(out[0, 0]), float(m[0, :3] @ v[0, :3] + m[0, 3]), rel_tol=1e-5, abs_tol=1e-5)
