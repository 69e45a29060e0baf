"""Cosine pre-weighting (fan and cone) and per-view source heights (z-offset
and helical cone orbits) on the GPU against the FP64 oracle, through the C
ABI.  Tolerances as everywhere: relative L2 <= 1e-4, adjoint dot-product
mismatch <= 1e-5."""
from __future__ import annotations

import math

import numpy as np
import pytest
import torch

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import _lib
from fanbeamctrecon_tensorflowop_gb300.batch import UnevenBatch
from fanbeamctrecon_tensorflowop_gb300.ops import ConePlan, FanPlan
import geometries as G

pytestmark = pytest.mark.gpu

TOL = 1e-4
DOT_TOL = 1e-5


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)


def _np(t):
    torch.cuda.synchronize()
    return t.detach().float().cpu().numpy().astype(np.float64)


def _dot(ax, y, x, aty):
    return abs(float(np.vdot(ax, y)) - float(np.vdot(x, aty))) / (
        np.linalg.norm(ax) * np.linalg.norm(y))


@pytest.mark.parametrize("short_scan", [False, True])
def test_fan_cosine_weighted_fbp(cuda, orc, short_scan):
    p, a = (G.short_scan(n=64, views=120, cols=192, pixel=4.0, dcol=4.0 * G.DCOL, shift=0.75)
            if short_scan else G.small(n=50, ny=38, shift=1.5, views=72, cols=100))
    plan = FanPlan(p, a, device=cuda, cosine_weight=True, short_scan=short_scan)
    g = orc.decode(p)
    rng = np.random.default_rng(3)
    y = rng.uniform(0, 1, (2, g.n_views, g.n_cols)).astype(np.float32)
    x = rng.standard_normal((2, g.ny, g.nx)).astype(np.float32)
    kw = dict(short_scan=short_scan, cosine=True)
    for got, ref in ((plan.fbp(_t(y, cuda)), orc.fbp_fan(g, a, y, **kw)),
                     (plan.fdk_bp(_t(y, cuda)), orc.fdk_bp(g, a, y, **kw))):
        assert rel_l2(_np(got), ref) <= TOL, rel_l2(_np(got), ref)
    ax = _np(plan.fbp_adjoint(_t(x, cuda)))
    assert rel_l2(ax, orc.fbp_fan_adjoint(g, a, x, **kw)) <= TOL
    assert _dot(ax, y, x, _np(plan.fbp(_t(y, cuda)))) <= DOT_TOL


def _helix(g, a, nz, pitch_frac=0.8):
    return (pitch_frac * g.dz * nz * (a - a[0]) / (2 * math.pi) - 0.4 * g.dz * nz).astype(
        np.float32)


@pytest.mark.parametrize("orbit", ["z_offset", "helix"])
@pytest.mark.parametrize("cosine", [False, True])
def test_cone_orbits(cuda, orc, orbit, cosine):
    p, a, nr, nz = G.cone_small(n=27, views=31, cols=57, n_rows=7, nz=9, pixel=6.6)
    g = orc.decode(p)
    zs = (np.full(g.n_views, 1.7 * g.dz, np.float32) if orbit == "z_offset"
          else _helix(g, a, nz))
    plan = ConePlan(p, a, nr, nz, device=cuda, cosine_weight=cosine, source_z=zs)
    rng = np.random.default_rng(6)
    vol = rng.uniform(0, 1, (2, nz, g.ny, g.nx)).astype(np.float32)
    got = _np(plan.fp_cone(_t(vol, cuda)))
    ref = orc.cone_fp(g, nr, nz, a, vol, source_z=zs)
    assert rel_l2(got, ref) <= TOL, ("fp", rel_l2(got, ref))
    y = ref.astype(np.float32)
    got = _np(plan.cone_bp(_t(y, cuda)))
    ref = orc.cone_bp(g, nr, nz, a, y, source_z=zs)
    assert rel_l2(got, ref) <= TOL, ("bp", rel_l2(got, ref))
    got = _np(plan.fdk(_t(y, cuda)))
    ref = orc.fdk_cone(g, nr, nz, a, y, cosine=cosine, source_z=zs)
    assert rel_l2(got, ref) <= TOL, ("fdk", rel_l2(got, ref))
    x = rng.standard_normal((2, nz, g.ny, g.nx)).astype(np.float32)
    ax = _np(plan.fdk_adjoint(_t(x, cuda)))
    ref = orc.fdk_cone_adjoint(g, nr, nz, a, x, cosine=cosine, source_z=zs)
    assert rel_l2(ax, ref) <= TOL, ("fdk_adjoint", rel_l2(ax, ref))
    yy = rng.standard_normal((2, g.n_views, nr, g.n_cols)).astype(np.float32)
    ax = _np(plan.fdk_adjoint(_t(x, cuda)))
    assert _dot(ax, yy, x, _np(plan.fdk(_t(yy, cuda)))) <= DOT_TOL


def test_source_z_validation(cuda):
    p, a, nr, nz = G.cone_small()
    with pytest.raises(ValueError):
        ConePlan(p, a, nr, nz, device=cuda, source_z=np.zeros(3, np.float32))
    zs = np.zeros(len(a), np.float32)
    zs[1] = np.nan
    with pytest.raises(RuntimeError):
        ConePlan(p, a, nr, nz, device=cuda, source_z=zs)
    # zero heights are the plain circular orbit
    plain = ConePlan(p, a, nr, nz, device=cuda)
    zero = ConePlan(p, a, nr, nz, device=cuda, source_z=np.zeros(len(a), np.float32))
    v = torch.rand((1, nz, plain.geom.ny, plain.geom.nx), device=cuda)
    assert torch.equal(plain.fp_cone(v), zero.fp_cone(v))
    assert torch.equal(plain.fdk(plain.fp_cone(v)), zero.fdk(zero.fp_cone(v)))


def test_cosine_plans_in_uneven_batch(cuda):
    items, ref = [], []
    for k, op in enumerate(("fbp", "fbp_adjoint", "fbp")):
        p, a = G.uneven(k, scale=4)
        plan = FanPlan(p, a, device=cuda, cosine_weight=(k != 2))
        x = (torch.rand(plan.image_shape, device=cuda) if op == "fbp_adjoint"
             else torch.rand(plan.sino_shape, device=cuda))
        y = torch.full(plan.sino_shape if op == "fbp_adjoint" else plan.image_shape,
                       float("nan"), device=cuda)
        items.append((plan, op, x, y))
        ref.append({"fbp": plan.fbp, "fbp_adjoint": plan.fbp_adjoint}[op](x)[0])
    UnevenBatch(items).run()
    for (plan, op, x, y), want in zip(items, ref):
        assert rel_l2(_np(y), _np(want)) <= 1e-5, op
