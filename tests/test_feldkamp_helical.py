"""Feldkamp cosine pre-weighting and per-view source heights (z-offset and
helical orbits) in the oracle, against known answers (CPU only).

The reference's FBP weights by 1/L^2 only (FBP/transform.cu:61-89) and its
view record's source height is always 0 (FDK/GPURecon_GPU.cu:226, fields of
FDK/GPURecon_GPU.h:27-33); both options are off by default."""
from __future__ import annotations

import math

import numpy as np
import pytest

from fanbeamctrecon_tensorflowop_gb300 import phantom
import geometries as G


def test_cosine_table(orc):
    p, a, nr, nz = G.cone_small(n=20, views=12, cols=40, n_rows=6, nz=5)
    g = orc.decode(p)
    w = orc.cosine_weights(g, nr, cone=True)
    gam = g.left + (np.arange(g.n_cols) + 0.5 - g.shift) * g.dcol
    h = g.det_bottom + (np.arange(nr) + 0.5) * g.drow
    np.testing.assert_allclose(w, np.cos(gam)[None, :] * (g.sdd / np.hypot(g.sdd, h))[:, None],
                               rtol=1e-14)
    np.testing.assert_allclose(orc.cosine_weights(g, 1, cone=False)[0], np.cos(gam), rtol=1e-15)


@pytest.mark.parametrize("cx,rad", [(0.0, 0.6), (0.45, 0.35)])
def test_cosine_weighted_fbp_recovers_disc_closely(orc, cx, rad):
    """With cos(gamma) the equiangular FBP is the textbook one and recovers a
    uniform disc to ~1e-4; the reference's unweighted FBP is off by ~0.5%."""
    n, pix, views, cols = 128, 2.0, 360, 320
    p = G.fan_param16(sdd=G.SDD, sid=G.SID, n_views=views, n_cols=cols, n=n, pixel_mm=pix,
                      dcol_rad=1.5 * G.DCOL)
    a = G.angle(views, 0.0)
    g = orc.decode(p)
    mu, R, X = 0.02, rad * g.rfov, cx * g.rfov
    p0, u = phantom.fan_rays(g.sid, a, g.left, g.dcol, g.n_cols)
    sino = phantom.ellipse_line_integrals(np.array([[X, 0.0, R, R, 0.0, mu]]), p0, u)
    x = g.xmin + g.dx * (np.arange(n) + 0.5)
    interior = np.sqrt((x[None, :] - X) ** 2 + x[:, None] ** 2) < 0.7 * R
    weighted = orc.fbp_fan(g, a, sino, cosine=True)[0]
    plain = orc.fbp_fan(g, a, sino)[0]
    err_w = np.abs(weighted[interior] / mu - 1).max()
    err_p = np.abs(plain[interior] / mu - 1).max()
    assert err_w < 5e-4 and err_p > 10 * err_w


def _padded_volume(g, nz, pad, seed=0):
    v = np.zeros((nz, g.ny, g.nx))
    rng = np.random.default_rng(seed)
    for k in range(pad, nz - pad):
        v[k] = phantom.ellipse_phantom(g.nx, float(g.dx), seed=seed + k, ny=g.ny) * (
            1.0 + 0.2 * rng.standard_normal())
    return v


def test_source_height_shift_equals_volume_shift(orc):
    """A source raised by m slices sees the volume as if it had moved down by
    m slices (edges zero, so the z clamp plays no part), for FP and BP."""
    p, a, nr, nz = G.cone_small(n=24, views=10, cols=48, n_rows=10, nz=12)
    g = orc.decode(p)
    m = 2
    vol = _padded_volume(g, nz, pad=m + 1)
    zs = np.full(g.n_views, m * g.dz, np.float32)
    shifted = np.zeros_like(vol)
    shifted[: nz - m] = vol[m:]
    np.testing.assert_allclose(orc.cone_fp(g, nr, nz, a, vol, source_z=zs),
                               orc.cone_fp(g, nr, nz, a, shifted), rtol=1e-9, atol=1e-12)
    y = orc.cone_fp(g, nr, nz, a, vol)
    up = orc.cone_bp(g, nr, nz, a, y, source_z=zs)[0]
    base = orc.cone_bp(g, nr, nz, a, y)[0]
    np.testing.assert_allclose(up[m:], base[: nz - m], rtol=1e-9, atol=1e-12)


def test_helical_adjoint_identities(orc):
    p, a, nr, nz = G.cone_small(n=20, views=16, cols=40, n_rows=6, nz=7)
    g = orc.decode(p)
    zs = (0.8 * g.dz * nz * (a - a[0]) / (2 * math.pi) - 0.4 * g.dz * nz).astype(np.float32)
    rng = np.random.default_rng(4)
    x = rng.standard_normal((1, nz, g.ny, g.nx))
    y = rng.standard_normal((1, g.n_views, nr, g.n_cols))
    pairs = [
        (orc.cone_bp_transpose(g, nr, nz, a, x, source_z=zs),
         orc.cone_bp(g, nr, nz, a, y, source_z=zs)),
        (orc.fdk_cone_adjoint(g, nr, nz, a, x, cosine=True, source_z=zs),
         orc.fdk_cone(g, nr, nz, a, y, cosine=True, source_z=zs)),
    ]
    for ax, aty in pairs:
        lhs, rhs = float(np.vdot(ax, y)), float(np.vdot(x, aty))
        assert abs(lhs - rhs) <= 1e-12 * np.linalg.norm(ax) * np.linalg.norm(y)
