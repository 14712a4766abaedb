"""CPU oracle of the vertex shaders -- test infrastructure only.

Restates in numpy float32 (every operation rounded on its own, as the GPU's
explicitly rounded intrinsics) the reference's vertexShader_gouraud and
vertexShader_texPhong (test/shader/Shaders.cu:37-108) as
cudaraster-linux_gb300/csrc/vertex.cu evaluates them: the framework's vector
and matrix C (src/framework/base/Math.hpp:112-202, 990-1001 -- sums from zero,
left to right; normalized(v) = v * (1 * rcp(length)); rcp(0) = 0), IEEE sqrt,
and the exact power pow_exact in place of the reference's fast-math powf: log2
from the atanh series of the mantissa in [sqrt(1/2), sqrt(2)], exp2 from the
Taylor series of e^(f ln 2) around f = 1/2, with the same float32 constants
and the same order of operations.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32

LOG2_COEFS = [f32("0.26230818"), f32("0.3205989"), f32("0.41219857"), f32("0.57707804"), f32("0.9617967"),
              f32("2.88539")]
EXP2_COEFS = [f32("1.0178086e-07"), f32("1.3215487e-06"), f32("1.5252734e-05"), f32("1.540353e-04"),
              f32("1.3333558e-03"), f32("9.618129e-03"), f32("5.550411e-02"), f32("2.402265e-01"),
              f32("6.931472e-01"), f32("1.0")]
SQRT2 = f32("1.4142135")
INF = f32(np.inf)


def _pow2(e: np.ndarray) -> np.ndarray:
    """2^e as float32 for integer e in [-126, 127]."""
    return ((e.astype(np.int64) + 127) << 23).astype(np.uint32).view(np.float32)


def log2_exact(x: np.ndarray) -> np.ndarray:
    """log2 of positive finite float32 values (vertex.cu log2Exact)."""
    x = np.asarray(x, np.float32).copy()
    b = x.view(np.uint32)
    k = np.zeros(x.shape, np.int64)
    sub = (b >> 23) == 0
    if sub.any():
        x[sub] = x[sub] * f32(16777216.0)
        k[sub] = -24
    b = x.view(np.uint32)
    k = k + (b >> 23).astype(np.int64) - 127
    m = ((b & np.uint32(0x7FFFFF)) | np.uint32(0x3F800000)).view(np.float32)
    big = m > f32("1.41421354")
    m = np.where(big, m * f32(0.5), m).astype(np.float32)
    k = k + big
    t = (m - f32(1.0)) / (m + f32(1.0))
    t2 = t * t
    p = np.full(x.shape, LOG2_COEFS[0], np.float32)
    for c in LOG2_COEFS[1:]:
        p = p * t2 + c
    return (k.astype(np.float32) + t * p).astype(np.float32)


def exp2_exact(z: np.ndarray) -> np.ndarray:
    """2^z for float32 z (vertex.cu exp2Exact)."""
    z = np.asarray(z, np.float32)
    out = np.empty(z.shape, np.float32)
    nan = z != z
    hi = z >= f32(128.0)
    lo = ~(z > f32(-150.0)) & ~nan
    ok = ~(nan | hi | lo)
    zz = np.where(ok, z, f32(0.0)).astype(np.float32)
    n = np.floor(zz).astype(np.float32)
    f = (zz - n) - f32(0.5)
    p = np.full(z.shape, EXP2_COEFS[0], np.float32)
    for c in EXP2_COEFS[1:]:
        p = p * f + c
    p = p * SQRT2
    ni = n.astype(np.int64)
    small = ni < -126
    p = np.where(small, p * _pow2(np.full(z.shape, -64)), p).astype(np.float32)
    ni = np.where(small, ni + 64, ni)
    r = (p * _pow2(np.clip(ni, -126, 127))).astype(np.float32)
    out[ok] = r[ok]
    out[nan] = z[nan]
    out[hi] = INF
    out[lo] = f32(0.0)
    return out


def pow_exact(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """x^y for x >= 0 (vertex.cu powExact)."""
    x = np.asarray(x, np.float32)
    y = np.asarray(y, np.float32)
    x, y = np.broadcast_arrays(x, y)
    out = np.empty(x.shape, np.float32)
    y0 = y == f32(0.0)
    nonpos = ~(x > f32(0.0)) & ~y0
    xinf = (x == INF) & ~y0
    rest = ~(y0 | nonpos | xinf)
    out[y0] = f32(1.0)
    out[nonpos] = np.where(y[nonpos] > f32(0.0), f32(0.0), INF)
    out[xinf] = np.where(y[xinf] > f32(0.0), INF, f32(0.0))
    if rest.any():
        out[rest] = exp2_exact(y[rest] * log2_exact(x[rest]))
    return out


def _mat_vec(m: np.ndarray, v: np.ndarray, rows: int) -> np.ndarray:
    """Rows of m (row-major, cols = v's width) times v, each sum from zero left to right."""
    cols = v.shape[1]
    out = np.empty((v.shape[0], rows), np.float32)
    for i in range(rows):
        acc = np.zeros(v.shape[0], np.float32)
        for j in range(cols):
            acc = acc + m[i * cols + j] * v[:, j]
        out[:, i] = acc
    return out


def _dot3(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    r = np.zeros(a.shape[0], np.float32) + a[:, 0] * b[:, 0]
    r = r + a[:, 1] * b[:, 1]
    return r + a[:, 2] * b[:, 2]


def _normalize3(v: np.ndarray) -> np.ndarray:
    length = np.sqrt(_dot3(v, v))
    with np.errstate(divide="ignore"):
        r = np.where(length != f32(0.0), f32(1.0) / length, f32(0.0)).astype(np.float32)
    s = f32(1.0) * r
    return (v * s[:, None]).astype(np.float32)


def vertex_passthrough(model, mvp) -> np.ndarray:
    """vertexShader_passthrough (test/shader/PassThrough.cu:16-35): clip = MVP * (xyz, 1),
    each row summed left to right from zero (Math.hpp:990-1001)."""
    m = np.asarray(mvp, dtype=np.float32).reshape(4, 4)
    v = np.asarray(model, dtype=np.float32)
    out = np.empty((v.shape[0], 4), np.float32)
    for r in range(4):
        acc = np.zeros(v.shape[0], np.float32)
        for c in range(3):
            acc = acc + m[r, c] * v[:, c]
        out[:, r] = acc + m[r, 3] * np.float32(1.0)
    return out


def vertex_gouraud(vertices, pos_to_clip, pos_to_camera, normal_to_camera, materials, material_idx):
    """InputVertex records [N, 8] -> GouraudVertex records [N, 8]."""
    v = np.asarray(vertices, np.float32)
    pc, pk, nk = (np.asarray(m, np.float32).reshape(-1) for m in (pos_to_clip, pos_to_camera, normal_to_camera))
    mats = np.asarray(materials, np.float32)
    idx = np.clip(np.asarray(material_idx, np.int64), 0, mats.shape[0] - 1)
    pos = np.concatenate([v[:, 0:3], np.ones((v.shape[0], 1), np.float32)], axis=1)
    camera_pos = _mat_vec(pk, pos, 3)
    camera_normal = _mat_vec(nk, v[:, 3:6], 3)
    clip = _mat_vec(pc, pos, 4)
    mat = mats[idx]
    I = _normalize3(camera_pos)
    N = _normalize3(camera_normal)
    dot_in = _dot3(I, N)
    twice = dot_in * f32(2.0)
    R = (I - N * twice[:, None]).astype(np.float32)
    diffuse_coef = np.fmax(-dot_in, f32(0.0)) * f32(0.75) + f32(0.25)
    specular_coef = pow_exact(np.fmax(-_dot3(I, R), f32(0.0)), mat[:, 7])
    color = (mat[:, 0:3] * diffuse_coef[:, None] + mat[:, 4:7] * specular_coef[:, None]).astype(np.float32)
    return np.concatenate([clip, color, mat[:, 3:4]], axis=1).astype(np.float32)


def vertex_tex_phong(vertices, pos_to_clip, pos_to_camera, normal_to_camera):
    """InputVertex records [N, 8] -> ShadedVertex_texPhong records [N, 16]."""
    v = np.asarray(vertices, np.float32)
    pc, pk, nk = (np.asarray(m, np.float32).reshape(-1) for m in (pos_to_clip, pos_to_camera, normal_to_camera))
    n = v.shape[0]
    pos = np.concatenate([v[:, 0:3], np.ones((n, 1), np.float32)], axis=1)
    out = np.zeros((n, 16), np.float32)
    out[:, 0:4] = _mat_vec(pc, pos, 4)
    out[:, 4:8] = _mat_vec(pk, pos, 4)
    out[:, 8:11] = _mat_vec(nk, v[:, 3:6], 3)
    out[:, 12:14] = v[:, 6:8]
    out[:, 15] = f32(1.0)
    return out
