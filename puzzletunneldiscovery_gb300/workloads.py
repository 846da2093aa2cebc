"""Seeded synthetic meshes and query batches for the collision-query path.

The reference measures its planner on puzzle meshes loaded from OBJ files
(``res/``) and on random states produced by ``src/GP/pipeline/uw_random.py``
(Shoemake quaternions, ``random_state`` at lines 8-17) and random segments
from ``src/GP/pipeline/touchq_util.py:8-13``.  No benchmark data set ships
with it, so these generators build the same kinds of inputs from seeds:

* ``torus`` -- (R, r, nu x nv) tube mesh, 2 * nu * nv triangles;
* ``interlocking_tori`` -- env torus plus the same torus rotated 90 degrees
  about x and offset by 1 along x (the classic two-ring puzzle);
* ``torus_knot`` -- a (p, q) torus-knot tube;
* ``perforated_plate`` -- a flat grid plate with circular holes whose
  vertices are displaced by Perlin's improved noise (Perlin 2002);
* ``uniform_states`` / ``segment_batch`` -- Shoemake-uniform rotations and
  uniform / Gaussian translations, expressed in the unit frame.

Every array is numpy; vertices are float32 (as loaded meshes are) and states
are float64 7-vectors ``[x, y, z, w, qx, qy, qz]``.
"""
from __future__ import annotations

import math

import numpy as np


def torus(R: float = 1.0, r: float = 0.25, nu: int = 64, nv: int = 32):
    """Torus in the xy-plane centred at the origin: (V float32 [nu*nv, 3], F uint32 [2*nu*nv, 3])."""
    iu, iv = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    u = 2.0 * np.pi * iu / nu
    v = 2.0 * np.pi * iv / nv
    x = (R + r * np.cos(v)) * np.cos(u)
    y = (R + r * np.cos(v)) * np.sin(u)
    z = r * np.sin(v)
    V = np.stack([x, y, z], axis=-1).reshape(-1, 3).astype(np.float32)
    idx = lambda i, j: (i % nu) * nv + (j % nv)  # noqa: E731
    F = []
    for i in range(nu):
        for j in range(nv):
            a, b, c, d = idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)
            F.append((a, b, c))
            F.append((a, c, d))
    return V, np.asarray(F, dtype=np.uint32)


def interlocking_tori(R: float = 1.0, r: float = 0.25, nu: int = 64, nv: int = 32):
    """Env torus and a robot torus rotated 90 degrees about x, offset +1 along x.

    The rotation (x, y, z) -> (x, -z, y) is applied as an exact permutation so
    the robot mesh carries no trigonometric rounding.
    """
    Ve, Fe = torus(R, r, nu, nv)
    Vr = np.empty_like(Ve)
    Vr[:, 0] = Ve[:, 0] + np.float32(1.0)
    Vr[:, 1] = -Ve[:, 2]
    Vr[:, 2] = Ve[:, 1]
    return Ve, Fe.copy(), Vr, Fe.copy()


def torus_knot(p: int = 2, q: int = 3, nu: int = 256, nv: int = 16,
               R: float = 1.0, r: float = 0.4, tube: float = 0.1):
    """(p, q) torus-knot tube with nu samples along the knot and nv around the tube."""
    t = 2.0 * np.pi * np.arange(nu) / nu

    def curve(tt):
        rr = R + r * np.cos(q * tt)
        return np.stack([rr * np.cos(p * tt), rr * np.sin(p * tt), r * np.sin(q * tt)], axis=-1)

    c = curve(t)
    dc = curve(t + 1e-4) - curve(t - 1e-4)
    T = dc / np.linalg.norm(dc, axis=-1, keepdims=True)
    up = np.array([0.0, 0.0, 1.0])
    N = np.cross(T, up)
    N /= np.linalg.norm(N, axis=-1, keepdims=True)
    B = np.cross(T, N)
    a = 2.0 * np.pi * np.arange(nv) / nv
    V = (c[:, None, :] + tube * (np.cos(a)[None, :, None] * N[:, None, :]
                                 + np.sin(a)[None, :, None] * B[:, None, :]))
    V = V.reshape(-1, 3).astype(np.float32)
    F = []
    for i in range(nu):
        for j in range(nv):
            a0 = i * nv + j
            b0 = ((i + 1) % nu) * nv + j
            c0 = ((i + 1) % nu) * nv + (j + 1) % nv
            d0 = i * nv + (j + 1) % nv
            F.append((a0, b0, c0))
            F.append((a0, c0, d0))
    return V, np.asarray(F, dtype=np.uint32)


def _perlin_perm(rng):
    p = rng.permutation(256)
    return np.concatenate([p, p]).astype(np.int64)


def perlin2(x, y, perm):
    """Perlin's improved gradient noise (2002) evaluated in 2-D (z = 0)."""
    def fade(t):
        return t * t * t * (t * (t * 6 - 15) + 10)

    def grad(h, x, y):
        h = h & 15
        u = np.where(h < 8, x, y)
        v = np.where(h < 4, y, np.where((h == 12) | (h == 14), x, 0.0))
        return np.where(h & 1, -u, u) + np.where(h & 2, -v, v)

    xi = np.floor(x).astype(np.int64) & 255
    yi = np.floor(y).astype(np.int64) & 255
    xf = x - np.floor(x)
    yf = y - np.floor(y)
    u, v = fade(xf), fade(yf)
    aa = perm[perm[xi] + yi]
    ab = perm[perm[xi] + yi + 1]
    ba = perm[perm[xi + 1] + yi]
    bb = perm[perm[xi + 1] + yi + 1]
    x1 = grad(aa, xf, yf) + u * (grad(ba, xf - 1, yf) - grad(aa, xf, yf))
    x2 = grad(ab, xf, yf - 1) + u * (grad(bb, xf - 1, yf - 1) - grad(ab, xf, yf - 1))
    return x1 + v * (x2 - x1)


def perforated_plate(n: int = 400, extent: float = 2.0, holes: int = 25,
                     rmin: float = 0.1, rmax: float = 0.3, amp: float = 0.01,
                     seed: int = 0):
    """Flat n x n grid plate over [-extent, extent]^2 with circular holes.

    Grid cells whose centre falls inside a hole are dropped; z = amp * Perlin
    noise.  About 2 * n * n triangles minus the holes (~320k at n = 400).
    """
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-extent + rmax, extent - rmax, size=(holes, 2))
    radii = rng.uniform(rmin, rmax, size=holes)
    perm = _perlin_perm(rng)
    g = np.linspace(-extent, extent, n + 1)
    X, Y = np.meshgrid(g, g, indexing="ij")
    Z = amp * perlin2(X * 2.0 + 0.5, Y * 2.0 + 0.5, perm)
    V = np.stack([X, Y, Z], axis=-1).reshape(-1, 3).astype(np.float32)
    cx = 0.5 * (g[:-1, None] + g[1:, None]) * np.ones((1, n))
    cy = 0.5 * (g[None, :-1] + g[None, 1:]) * np.ones((n, 1))
    keep = np.ones((n, n), dtype=bool)
    for (hx, hy), hr in zip(centers, radii):
        keep &= (cx - hx) ** 2 + (cy - hy) ** 2 > hr * hr
    ii, jj = np.nonzero(keep)
    a = ii * (n + 1) + jj
    b = (ii + 1) * (n + 1) + jj
    c = (ii + 1) * (n + 1) + jj + 1
    d = ii * (n + 1) + jj + 1
    F = np.concatenate([np.stack([a, b, c], -1), np.stack([a, c, d], -1)], axis=0)
    used = np.unique(F)
    remap = np.full(V.shape[0], -1, dtype=np.int64)
    remap[used] = np.arange(used.size)
    return V[used], remap[F].astype(np.uint32), (centers, radii)


def shoemake_quaternions(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform unit quaternions, w-first, Shoemake's subgroup algorithm (1992).

    Same component order as uw_random.random_state (uw_random.py:11-15).
    """
    u1, u2, u3 = rng.random((3, n))
    a = np.sqrt(1.0 - u1)
    b = np.sqrt(u1)
    return np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                     b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)], axis=-1)


def uniform_states(n: int, lo, hi, scale: float, seed: int = 0) -> np.ndarray:
    """n states: translation uniform in the world box [lo, hi]^3, mapped to the
    unit frame by the scene scale; rotation Shoemake-uniform."""
    rng = np.random.default_rng(seed)
    lo = np.broadcast_to(np.asarray(lo, dtype=np.float64), (3,))
    hi = np.broadcast_to(np.asarray(hi, dtype=np.float64), (3,))
    t = rng.uniform(lo, hi, size=(n, 3))
    q = shoemake_quaternions(rng, n)
    return np.concatenate([t * scale, q], axis=1)


def _quat_mul(a, b):
    aw, ax, ay, az = a[..., 0], a[..., 1], a[..., 2], a[..., 3]
    bw, bx, by, bz = b[..., 0], b[..., 1], b[..., 2], b[..., 3]
    return np.stack([aw * bw - ax * bx - ay * by - az * bz,
                     aw * bx + ax * bw + ay * bz - az * by,
                     aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw], axis=-1)


def segment_batch(n: int, lo, hi, scale: float, sigma_t: float = 0.3,
                  max_angle: float = math.pi, seed: int = 0):
    """Segments: start as ``uniform_states``; end = start + N(0, sigma_t^2) world
    translation and a rotation by U[0, max_angle] about a uniform axis applied
    on the left (as pyosr.apply does, osr_state.cc:244-259)."""
    q0 = uniform_states(n, lo, hi, scale, seed)
    rng = np.random.default_rng(seed + 1_000_003)
    dt = rng.normal(0.0, sigma_t, size=(n, 3)) * scale
    ang = rng.uniform(0.0, max_angle, size=n)
    axis = rng.normal(size=(n, 3))
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    dq = np.concatenate([np.cos(ang / 2)[:, None], np.sin(ang / 2)[:, None] * axis], axis=1)
    q1 = np.empty_like(q0)
    q1[:, :3] = q0[:, :3] + dt
    q1[:, 3:] = _quat_mul(dq, q0[:, 3:])
    return q0, q1


def cfg_interlocking_tori():
    """Env/robot meshes of the interlocking-tori workload (4096 + 4096 triangles)."""
    return interlocking_tori(1.0, 0.25, 64, 32)


def cfg_plate_knot(n: int = 400, seed: int = 0):
    """Perforated plate (about 320k triangles) and a (2,3) torus knot (8192 triangles)."""
    Ve, Fe, _ = perforated_plate(n=n, seed=seed)
    Vr, Fr = torus_knot(2, 3, 256, 16)
    return Ve, Fe, Vr, Fr
