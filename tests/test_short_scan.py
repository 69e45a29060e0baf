"""Short-scan (Parker-weighted) reconstruction: the oracle's weights and
short-scan FBP against the geometry and analytic known answers (CPU only).

The reference's config carries a ParkWeighting switch (config.py:24) and its
FDK header a commented-out ApplyParkerWeighting (FDK/GPURecon_GPU.h:53), but
no reference op applies it; these tests pin the restatement on its defining
property (conjugate rays sum to one) and on reconstructions of known
phantoms."""
from __future__ import annotations

import math

import numpy as np
import pytest

from fanbeamctrecon_tensorflowop_gb300 import phantom
import geometries as G


def _gamma_of(g, beta, x, y):
    """Fan angle of the ray through (x, y) at view angle beta, by the
    backprojector's convention (BP/transform.cu:76-92)."""
    c, s = -math.cos(beta), -math.sin(beta)
    U = g.sid + x * c + y * s
    t = -x * s + y * c
    return math.atan2(t, U)


def test_conjugate_ray_of_this_geometry(orc):
    """The line through a point seen at (beta, gamma) is seen again at
    (beta + pi + 2 gamma, -gamma): the form the weights are built on."""
    p, _ = G.small()
    g = orc.decode(p)
    rng = np.random.default_rng(3)
    for _ in range(200):
        beta = rng.uniform(0, 2 * math.pi)
        r, phi = g.rfov * math.sqrt(rng.uniform()), rng.uniform(0, 2 * math.pi)
        x, y = r * math.cos(phi), r * math.sin(phi)
        gam = _gamma_of(g, beta, x, y)
        bc = beta + math.pi + 2.0 * gam
        gc = _gamma_of(g, bc, x, y)
        assert abs(gc + gam) < 1e-12
        # the same line: both source positions R (cos, sin) and the point
        # are collinear (U = R - x cos - y sin is the depth from the source)
        s1 = np.array([g.sid * math.cos(beta), g.sid * math.sin(beta)])
        s2 = np.array([g.sid * math.cos(bc), g.sid * math.sin(bc)])
        d1, d2 = np.array([x, y]) - s1, np.array([x, y]) - s2
        assert abs(d1[0] * d2[1] - d1[1] * d2[0]) < 1e-9 * np.linalg.norm(d1) * np.linalg.norm(d2)


def test_parker_conjugate_weights_sum_to_one(orc):
    half = 0.2
    rng = np.random.default_rng(5)
    worst = 0.0
    for _ in range(5000):
        beta = rng.uniform(0.0, math.pi + 2 * half)
        gam = rng.uniform(-half * 0.999, half * 0.999)
        bc = beta + math.pi + 2 * gam
        if bc > math.pi + 2 * half:
            bc -= 2 * math.pi
        w = orc.parker_weight(beta, gam, half) + orc.parker_weight(bc, -gam, half)
        worst = max(worst, abs(w - 1.0))
    assert worst < 1e-12
    # zero outside the short-scan range, one in its redundancy-free middle
    assert orc.parker_weight(-1e-9, 0.0, half) == 0.0
    assert orc.parker_weight(math.pi + 2 * half + 1e-9, 0.0, half) == 0.0
    assert orc.parker_weight(math.pi / 2, 0.0, half) == 1.0


def test_parker_table_of_a_plan(orc):
    """The doubled table: 2 w(beta_v, gamma_i); the same acquisition listed in
    reverse order gives every measurement the same weight."""
    p, a = G.short_scan(n=32, views=40, cols=48)
    g = orc.decode(p)
    w = orc.parker_weights(g, a)
    half = g.n_cols * g.dcol / 2.0
    gam = g.left + (np.arange(g.n_cols) + 0.5 - g.shift) * g.dcol
    for v in (0, 7, 20, 39):
        beta = float(a[v]) - float(a[0])
        ref = [2.0 * orc.parker_weight(beta, float(gi), half) for gi in gam]
        np.testing.assert_allclose(w[v], ref, rtol=0, atol=1e-15)
    assert np.all(w[0] == 0.0)
    wr = orc.parker_weights(g, a[::-1].copy())
    np.testing.assert_allclose(wr[::-1], w, rtol=0, atol=1e-6)


def _disc(g, a, cx, cy, rad, mu):
    ell = np.array([[cx, cy, rad, rad, 0.0, mu]])
    p0, u = phantom.fan_rays(g.sid, a, g.left, g.dcol, g.n_cols)
    return phantom.ellipse_line_integrals(ell, p0, u)


@pytest.mark.parametrize("reverse", [False, True])
def test_short_scan_fbp_recovers_off_centre_disc(orc, reverse):
    """A Parker-weighted FBP of pi + fan-angle of exact projections recovers an
    off-centre disc to the discrete-FBP level; the unweighted one does not."""
    p, a = G.short_scan(views=200, reverse=reverse)
    g = orc.decode(p)
    mu, rad, cx, cy = 0.02, 0.35 * g.rfov, 0.2 * g.rfov, -0.1 * g.rfov
    sino = _disc(g, a, cx, cy, rad, mu)
    x = g.xmin + g.dx * (np.arange(g.nx) + 0.5)
    r = np.sqrt((x[None, :] - cx) ** 2 + (x[:, None] - cy) ** 2)
    interior = r < 0.7 * rad
    rec = orc.fbp_fan(g, a, sino, short_scan=True)[0]
    assert abs(rec[interior].mean() / mu - 1.0) < 0.005
    assert np.abs(rec[interior] / mu - 1.0).max() < 0.02
    plain = orc.fbp_fan(g, a, sino)[0]
    assert abs(plain[interior].mean() / mu - 1.0) > 0.3


def test_short_scan_adjoint_identities(orc):
    p, a = G.short_scan(n=36, views=30, cols=64)
    g = orc.decode(p)
    rng = np.random.default_rng(1)
    x = rng.standard_normal((2, g.ny, g.nx))
    y = rng.standard_normal((2, g.n_views, g.n_cols))
    ax, aty = orc.fbp_fan_adjoint(g, a, x, short_scan=True), orc.fbp_fan(g, a, y, short_scan=True)
    lhs, rhs = float(np.vdot(ax, y)), float(np.vdot(x, aty))
    assert abs(lhs - rhs) <= 1e-12 * np.linalg.norm(ax) * np.linalg.norm(y)
    nz, rows = 3, 4
    xc = rng.standard_normal((1, nz, g.ny, g.nx))
    yc = rng.standard_normal((1, g.n_views, rows, g.n_cols))
    axc = orc.fdk_cone_adjoint(g, rows, nz, a, xc, short_scan=True)
    atyc = orc.fdk_cone(g, rows, nz, a, yc, short_scan=True)
    lhs, rhs = float(np.vdot(axc, yc)), float(np.vdot(xc, atyc))
    assert abs(lhs - rhs) <= 1e-12 * np.linalg.norm(axc) * np.linalg.norm(yc)
