"""The FP64 oracle against exact and analytic known answers (CPU only).

These pin the restatement where no reference output exists: exact answers of
the discrete operators, analytic line integrals, adjoint identities and the
FDK-op / FBP-op equivalence the reference's one-row texture implies."""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import phantom
from fanbeamctrecon_tensorflowop_gb300.geometry import ray_table
import geometries as G


def test_fp_constant_image_is_sample_count(orc):
    """FP of an all-ones image is 0.125*dx*n exactly (bilinear of a constant is
    the constant; clamp keeps edge samples inside): the sample rule of
    FP/transform.cu:91-92,144."""
    p, a = G.small(n=48, views=36, cols=64)
    g = orc.decode(p)
    sino = orc.fp_fan(g, a, np.ones((g.ny, g.nx)))[0]
    _, ns = orc.ray_table(g, a)
    np.testing.assert_allclose(sino, 0.125 * g.dx * ns, rtol=1e-13, atol=0)
    # chord rule: n = floor(2 sqrt(r^2 - d^2) / 0.125), d = R/dx sin(gamma)
    gam = g.left + (np.arange(g.n_cols) + 0.5) * g.dcol
    d = g.sid / g.dx * np.sin(gam)
    h = (g.rfov / g.dx) ** 2 - d**2
    expect = np.where(h > 0, np.floor(2 * np.sqrt(np.maximum(h, 0)) / 0.125), 0)
    # identical for every view; allow a one-sample flip where the chord is
    # within rounding of a multiple of 0.125
    assert np.all(np.abs(ns - expect[None, :]) <= 1)
    assert np.mean(ns == expect[None, :]) > 0.999


def test_ray_table_library_equals_oracle(orc):
    """The library's host FP64 ray table (ct_fp_ray_table) has exactly the
    oracle's sample counts and its starts/steps to float rounding."""
    for p, a in (G.small(), G.config0(), G.small(n=50, ny=40, shift=1.5)):
        g = orc.decode(p)
        ray_o, ns_o = orc.ray_table(g, a)
        ray_l, ns_l = ray_table(p, a)
        np.testing.assert_array_equal(ns_l, ns_o)
        np.testing.assert_allclose(ray_l, ray_o, rtol=2e-7, atol=1e-6)
        # some rays must miss the FOV (zero samples) in these geometries
        assert (ns_o == 0).any() and (ns_o > 0).any()


def test_bp_constant_sinogram_counts_views(orc):
    """BP of an all-ones sinogram is n_views inside the FOV, 0 outside, when
    the detector covers the FOV (BP/transform.cu:80,88)."""
    p, a = G.small(n=40, views=30, cols=96)
    g = orc.decode(p)
    img = orc.bp_fan(g, a, np.ones((g.n_views, g.n_cols)))[0]
    x = g.xmin + g.dx * (np.arange(g.nx) + 0.5)
    y = g.ymin + g.dy * (np.arange(g.ny) + 0.5)
    inside = (x[None, :] ** 2 + y[:, None] ** 2) <= np.float64(g.rfov) ** 2
    np.testing.assert_array_equal(img, np.where(inside, float(g.n_views), 0.0))


def test_fp_matches_analytic_ellipse_integrals(orc):
    """FP of a finely sampled ellipse phantom against exact line integrals.
    The discrete projector's bias (pixelisation, the floor() sample rule,
    clamp at the FOV edge) keeps this at the percent level."""
    n, pix = 192, 1.4
    p = G.fan_param16(sdd=G.SDD, sid=G.SID, n_views=24, n_cols=192, n=n, pixel_mm=pix,
                      dcol_rad=2.5 * G.DCOL)
    a = G.angle(24, 0.0)
    g = orc.decode(p)
    ell = phantom.random_ellipses(g.rfov, seed=3)
    img = phantom.rasterize(ell, n, n, pix, pix, supersample=4)
    sino = orc.fp_fan(g, a, img)[0]
    p0, u = phantom.fan_rays(g.sid, a, g.left, g.dcol, g.n_cols)
    ana = phantom.ellipse_line_integrals(ell, p0, u)
    assert rel_l2(sino, ana) < 2e-2


def test_fbp_of_uniform_disc_recovers_value(orc):
    """FBP (reference Ram-Lak filter) of the exact projections of a uniform
    disc returns the disc's attenuation in its interior (to the few-percent
    level of a discrete equiangular FBP)."""
    n, pix = 128, 2.0
    views, cols = 360, 320  # +-14.5 deg of detector covers the 13.7 deg FOV
    p = G.fan_param16(sdd=G.SDD, sid=G.SID, n_views=views, n_cols=cols, n=n, pixel_mm=pix,
                      dcol_rad=1.5 * G.DCOL)
    a = G.angle(views, 0.0)
    g = orc.decode(p)
    mu, rad = 0.02, 0.6 * g.rfov
    ell = np.array([[0.0, 0.0, rad, rad, 0.0, mu]])
    p0, u = phantom.fan_rays(g.sid, a, g.left, g.dcol, g.n_cols)
    sino = phantom.ellipse_line_integrals(ell, p0, u)
    rec = orc.fbp_fan(g, a, sino)[0]
    x = g.xmin + g.dx * (np.arange(n) + 0.5)
    r = np.sqrt(x[None, :] ** 2 + x[:, None] ** 2)
    interior = r < 0.7 * rad
    assert abs(rec[interior].mean() / mu - 1.0) < 0.02
    assert np.abs(rec[interior] / mu - 1.0).max() < 0.08
    outside = rec[(r > 1.3 * rad) & (r < 0.95 * g.rfov)]
    assert np.abs(outside).mean() < 0.02 * mu and np.abs(outside).max() < 0.2 * mu


@pytest.mark.parametrize("shift", [0.0, 1.25])
def test_oracle_adjoint_identities(orc, shift):
    """<A x, y> = <x, A^T y> in FP64 for FP, BP (both weightings), FBP."""
    p, a = G.small(n=36, views=20, cols=64, shift=shift, ny=30)
    g = orc.decode(p)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((2, g.ny, g.nx))
    y = rng.standard_normal((2, g.n_views, g.n_cols))
    pairs = [
        (orc.fp_fan(g, a, x), orc.fp_fan_adjoint(g, a, y)),
        (orc.bp_fan_transpose(g, a, x), orc.bp_fan(g, a, y)),
        (orc.bp_fan_transpose(g, a, x, weighted=True), orc.bp_fan(g, a, y, weighted=True)),
        (orc.fbp_fan_adjoint(g, a, x), orc.fbp_fan(g, a, y)),
    ]
    for ax, aty in pairs:
        lhs = float(np.vdot(ax, y))
        rhs = float(np.vdot(x, aty))
        assert abs(lhs - rhs) <= 1e-12 * np.linalg.norm(ax) * np.linalg.norm(y)


def test_ramp_taps_follow_reference_formula(orc):
    """Taps of FBP/transform.cu:149-162 (Hsieh h'' form, 0.5 factor, scaled by
    R*dAngle*dCol) and their symmetry; Shepp-Logan taps are all nonzero."""
    p, a = G.small(cols=32)
    g = orc.decode(p)
    t = orc.ramp_taps(g, orc.RAMLAK)
    C = g.n_cols
    n = np.arange(-(C - 1), C)
    pi = float(np.float32(3.14159265359))
    scale = float(g.sid) * float(g.d_angle) * float(g.dcol)
    expect = np.where(n == 0, 0.5 / (4 * g.dcol**2),
                      np.where(n % 2 != 0, -0.5 / (pi**2 * np.sin(n * g.dcol) ** 2 + (n == 0)),
                               0.0)) * scale
    np.testing.assert_allclose(t, expect, rtol=1e-14, atol=0)
    np.testing.assert_array_equal(t, t[::-1])
    sl = orc.ramp_taps(g, orc.SHEPP_LOGAN)
    np.testing.assert_array_equal(sl, sl[::-1])
    assert np.all(sl != 0) and sl[C - 1] > 0 and np.all(sl[:C - 1] < 0)


def test_ramp_filter_is_middle_of_full_convolution(orc):
    """q = middle C samples of the full linear convolution (the ippsConv_32f
    + memcpy(pfBuffer + nCols - 1) of FBP/transform.cu:171-172)."""
    p, a = G.small(cols=40, views=3)
    g = orc.decode(p)
    rng = np.random.default_rng(1)
    rows = rng.standard_normal((3, g.n_cols))
    taps = orc.ramp_taps(g, orc.RAMLAK)
    full = np.stack([np.convolve(r, taps) for r in rows])
    np.testing.assert_allclose(orc.ramp_filter(g, rows), full[:, g.n_cols - 1:2 * g.n_cols - 1],
                               rtol=1e-12, atol=1e-12 * np.abs(full).max())


def test_fdk_op_equals_fbp_op_with_one_row(orc):
    """The FDK op's CB_EA kernel on a one-row view texture (FDK/FBP.cc:85,98)
    reduces to the 1/L^2-weighted fan FBP with detector shift."""
    p, a = G.fdk_driver(nview=40, nimg=32)
    g = orc.decode(p)
    rng = np.random.default_rng(2)
    y = rng.uniform(0, 1, (1, g.n_views, g.n_cols))
    np.testing.assert_allclose(orc.fdk_bp(g, a, y), orc.fbp_fan(g, a, y), rtol=1e-13, atol=1e-16)


def test_texture_emulation_bounds_reference_deviation(orc):
    """8-bit texture-filter weights move FP of a phantom by ~1e-4..1e-3
    relative: the reference's own outputs sit that far from exact bilinear,
    which is why parity is stated against the exact-weight oracle."""
    p, a = G.small(n=64, views=24, cols=96)
    g = orc.decode(p)
    img = phantom.ellipse_phantom(64, 2.8, seed=0)
    exact = orc.fp_fan(g, a, img)
    orc.set_texture_emulation(True)
    try:
        tex = orc.fp_fan(g, a, img)
    finally:
        orc.set_texture_emulation(False)
    d = rel_l2(tex, exact)
    assert 1e-6 < d < 1e-2


# ---- cone beam ---------------------------------------------------------------

def test_fdk_cone_one_row_one_slice_is_the_fdk_op(orc):
    """With nz = n_rows = 1 (FDK/FBP.cc:85,98) the cone FDK is the 2-D op."""
    p, a = G.fdk_driver(nview=40, nimg=32)
    g = orc.decode(p)
    y = np.random.default_rng(2).uniform(0, 1, (1, g.n_views, 1, g.n_cols))
    np.testing.assert_allclose(orc.fdk_cone(g, 1, 1, a, y)[:, 0], orc.fdk_bp(g, a, y[:, :, 0]),
                               rtol=1e-13, atol=1e-16)


def test_cone_adjoint_identities(orc):
    p, a, nr, nz = G.cone_small(n=20, views=12, cols=40, n_rows=6, nz=5)
    g = orc.decode(p)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((1, nz, g.ny, g.nx))
    y = rng.standard_normal((1, g.n_views, nr, g.n_cols))
    for ax, aty in ((orc.cone_bp_transpose(g, nr, nz, a, x), orc.cone_bp(g, nr, nz, a, y)),
                    (orc.fdk_cone_adjoint(g, nr, nz, a, x), orc.fdk_cone(g, nr, nz, a, y))):
        lhs, rhs = float(np.vdot(ax, y)), float(np.vdot(x, aty))
        assert abs(lhs - rhs) <= 1e-12 * np.linalg.norm(ax) * np.linalg.norm(y)


def test_cone_fp_known_answers(orc):
    """A constant volume projects to 0.125*dx*n*sqrt(1+(h_r/D)^2) (trilinear of
    a constant, clamp-to-edge in z); a z-invariant volume projects to the fan
    FP of its slice times the same stretch factor."""
    p, a, nr, nz = G.cone_small(n=24, views=10, cols=48, n_rows=8, nz=6)
    g = orc.decode(p)
    _, ns = orc.ray_table(g, a)
    h = g.det_bottom + (np.arange(nr) + 0.5) * g.drow
    stretch = np.sqrt(1 + (h / g.sdd) ** 2)
    ones = orc.cone_fp(g, nr, nz, a, np.ones((nz, g.ny, g.nx)))[0]
    np.testing.assert_allclose(ones, 0.125 * g.dx * ns[:, None, :] * stretch[None, :, None],
                               rtol=1e-12, atol=0)
    sl = phantom.ellipse_phantom(24, float(g.dx), seed=4).astype(np.float64)
    cyl = orc.cone_fp(g, nr, nz, a, np.repeat(sl[None], nz, axis=0))[0]
    fan = orc.fp_fan(g, a, sl)[0]
    np.testing.assert_allclose(cyl, fan[:, None, :] * stretch[None, :, None], rtol=1e-10,
                               atol=1e-12)
