"""Seeded synthetic phantoms and their analytic fan-beam line integrals.

The workloads use numpy ``default_rng(seed)`` ellipse phantoms: a water disc of
0.019/mm with radius 0.9*rFOV plus ``n_ellipses`` additive ellipses whose
centres lie within 0.8*rFOV, semi-axes in [0.05, 0.4]*rFOV, uniform rotation
and attenuation uniform in [-0.01, 0.03]/mm.  Images are point-sampled at the
pixel centres x = xmin + dx*(i + 1/2) of the reference geometry.
"""
from __future__ import annotations

import math

import numpy as np

WATER_MU = 0.019  # 1/mm


def random_ellipses(rfov: float, seed: int, n_ellipses: int = 10) -> np.ndarray:
    """Rows (cx, cy, a, b, theta, mu) in mm / rad / (1/mm); row 0 is the water disc."""
    rng = np.random.default_rng(seed)
    rows = [(0.0, 0.0, 0.9 * rfov, 0.9 * rfov, 0.0, WATER_MU)]
    for _ in range(n_ellipses):
        r = 0.8 * rfov * math.sqrt(rng.uniform())
        phi = rng.uniform(0.0, 2.0 * math.pi)
        a, b = rng.uniform(0.05 * rfov, 0.4 * rfov, size=2)
        theta = rng.uniform(0.0, math.pi)
        mu = rng.uniform(-0.01, 0.03)
        rows.append((r * math.cos(phi), r * math.sin(phi), a, b, theta, mu))
    return np.asarray(rows, dtype=np.float64)


def rasterize(ellipses: np.ndarray, nx: int, ny: int, dx: float, dy: float,
              supersample: int = 1) -> np.ndarray:
    """float32 [ny, nx] image: the sum of mu over ellipses covering each pixel
    centre (or the mean over supersample^2 sub-pixel points)."""
    xmin, ymin = -0.5 * nx * dx, -0.5 * ny * dy
    s = supersample
    off = (np.arange(s) + 0.5) / s
    xs = xmin + dx * (np.arange(nx)[:, None] + off[None, :]).reshape(-1)
    ys = ymin + dy * (np.arange(ny)[:, None] + off[None, :]).reshape(-1)
    X, Y = np.meshgrid(xs, ys)
    img = np.zeros_like(X)
    for cx, cy, a, b, th, mu in ellipses:
        c, sn = math.cos(th), math.sin(th)
        u = (X - cx) * c + (Y - cy) * sn
        v = -(X - cx) * sn + (Y - cy) * c
        img += mu * ((u / a) ** 2 + (v / b) ** 2 <= 1.0)
    if s > 1:
        img = img.reshape(ny, s, nx, s).mean(axis=(1, 3))
    return img.astype(np.float32)


def ellipse_phantom(n: int, pixel_mm: float, seed: int, n_ellipses: int = 10,
                    ny: int | None = None) -> np.ndarray:
    """The seeded 2-D phantom of the workloads, float32 [ny, n]."""
    ny = n if ny is None else ny
    rfov = n * pixel_mm / 2.0
    return rasterize(random_ellipses(rfov, seed, n_ellipses), n, ny, pixel_mm, pixel_mm)


def ellipsoid_phantom(n: int, nz: int, pixel_mm: float, dz_mm: float, seed: int,
                      n_ellipsoids: int = 12) -> np.ndarray:
    """The seeded 3-D phantom of the cone workload, float32 [nz, n, n]: a water
    cylinder (0.019/mm, radius 0.9*rFOV, 0.9 of the volume's height) plus
    ``n_ellipsoids`` additive ellipsoids -- centres within 0.8*rFOV in x-y and
    0.6 of the half-height in z, in-plane semi-axes in [0.05, 0.4]*rFOV, z
    semi-axis in [0.1, 0.5] of the half-height, uniform rotation about z,
    attenuation uniform in [-0.01, 0.03]/mm -- sampled at the voxel centres."""
    rng = np.random.default_rng(seed)
    rfov = n * pixel_mm / 2.0
    hz = nz * dz_mm / 2.0
    x = (np.arange(n) + 0.5) * pixel_mm - rfov
    z = (np.arange(nz) + 0.5) * dz_mm - hz
    X, Y = np.meshgrid(x, x)
    vol = np.zeros((nz, n, n), np.float64)
    cyl = (X ** 2 + Y ** 2 <= (0.9 * rfov) ** 2)
    vol[np.abs(z) <= 0.9 * hz] += WATER_MU * cyl
    for _ in range(n_ellipsoids):
        r = 0.8 * rfov * math.sqrt(rng.uniform())
        phi = rng.uniform(0.0, 2.0 * math.pi)
        cx, cy = r * math.cos(phi), r * math.sin(phi)
        cz = rng.uniform(-0.6, 0.6) * hz
        a, b = rng.uniform(0.05 * rfov, 0.4 * rfov, size=2)
        c = rng.uniform(0.1, 0.5) * hz
        th = rng.uniform(0.0, math.pi)
        mu = rng.uniform(-0.01, 0.03)
        cs, sn = math.cos(th), math.sin(th)
        q = (((X - cx) * cs + (Y - cy) * sn) / a) ** 2 + ((-(X - cx) * sn + (Y - cy) * cs) / b) ** 2
        for k in np.nonzero(np.abs(z - cz) <= c)[0]:
            vol[k] += mu * (q + ((z[k] - cz) / c) ** 2 <= 1.0)
    return vol.astype(np.float32)


def phantom_batch(batch: int, n: int, pixel_mm: float, seed0: int = 0) -> np.ndarray:
    """float32 [batch, n, n] with seeds seed0 .. seed0+batch-1."""
    return np.stack([ellipse_phantom(n, pixel_mm, seed0 + b) for b in range(batch)])


def ellipse_line_integrals(ellipses: np.ndarray, p0: np.ndarray, u: np.ndarray) -> np.ndarray:
    """Sum over ellipses of mu * chord length of the lines p0 + t*u (u unit).

    p0, u: [..., 2] arrays in mm.  Exact: each ellipse maps to the unit circle
    and the chord follows from the quadratic's discriminant."""
    out = np.zeros(p0.shape[:-1])
    for cx, cy, a, b, th, mu in ellipses:
        c, s = math.cos(th), math.sin(th)
        qx = (p0[..., 0] - cx) * c + (p0[..., 1] - cy) * s
        qy = -(p0[..., 0] - cx) * s + (p0[..., 1] - cy) * c
        ux = u[..., 0] * c + u[..., 1] * s
        uy = -u[..., 0] * s + u[..., 1] * c
        A = (ux / a) ** 2 + (uy / b) ** 2
        B = 2.0 * (qx * ux / a**2 + qy * uy / b**2)
        C0 = (qx / a) ** 2 + (qy / b) ** 2 - 1.0
        disc = B * B - 4.0 * A * C0
        out += mu * np.where(disc > 0, np.sqrt(np.maximum(disc, 0.0)) / A, 0.0)
    return out


def fan_rays(sid: float, angles: np.ndarray, left: float, dcol: float, n_cols: int):
    """Source points and unit directions of every (view, channel) ray in mm.

    Source at R(cos b, sin b); channel i at fan angle left + (i+1/2) dcol; the
    ray direction is -(cos(b+g), sin(b+g)) (towards the detector)."""
    b = np.asarray(angles, np.float64)[:, None]
    g = left + (np.arange(n_cols) + 0.5) * dcol
    th = b + g[None, :]
    p0 = np.stack([sid * np.cos(b) + 0 * th, sid * np.sin(b) + 0 * th], axis=-1)
    u = -np.stack([np.cos(th), np.sin(th)], axis=-1)
    return p0, u
