"""Cone-beam operators on the GPU against the FP64 oracle, through the C ABI.
Tolerance as for the fan-beam operators: relative L2 <= 1e-4, adjoint
dot-product mismatch <= 1e-5."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import _lib, phantom
from fanbeamctrecon_tensorflowop_gb300.ops import ConePlan, FanPlan
import geometries as G

pytestmark = pytest.mark.gpu

TOL = 1e-4
DOT_TOL = 1e-5


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)


def _np(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy().astype(np.float64)


def _vol(g, nz, batch, seed=0):
    out = []
    for b in range(batch):
        sl = phantom.ellipse_phantom(g.nx, float(g.dx), seed=seed + b, ny=g.ny)
        w = 1.0 + 0.3 * np.sin(np.linspace(0, 3, nz))[:, None, None]
        out.append(sl[None] * w)
    return np.stack(out).astype(np.float32)


CASES = {
    "small": lambda: G.cone_small(),
    "odd": lambda: G.cone_small(n=27, views=31, cols=57, n_rows=7, nz=9, pixel=6.6),
}


@pytest.fixture(scope="module", params=list(CASES))
def cone(request, cuda, orc):
    p, a, nr, nz = CASES[request.param]()
    plan = ConePlan(p, a, nr, nz, device=cuda)
    plan_sl = ConePlan(p, a, nr, nz, device=cuda, window=_lib.WINDOW_SHEPP_LOGAN)
    return p, a, nr, nz, plan, plan_sl, orc.decode(p)


def test_cone_fp(cone, cuda, orc):
    p, a, nr, nz, plan, _, g = cone
    x = _vol(g, nz, 2)
    got = _np(plan.fp_cone(_t(x, cuda)))
    ref = orc.cone_fp(g, nr, nz, a, x)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)


def test_cone_bp_and_fdk(cone, cuda, orc):
    p, a, nr, nz, plan, plan_sl, g = cone
    y = orc.cone_fp(g, nr, nz, a, _vol(g, nz, 2, seed=3))
    got = _np(plan.cone_bp(_t(y, cuda)))
    ref = orc.cone_bp(g, nr, nz, a, y)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)
    for pl, w in ((plan, orc.RAMLAK), (plan_sl, orc.SHEPP_LOGAN)):
        got = _np(pl.fdk(_t(y, cuda)))
        ref = orc.fdk_cone(g, nr, nz, a, y, w)
        assert rel_l2(got, ref) <= TOL, (w, rel_l2(got, ref))


def test_fdk_adjoint(cone, cuda, orc):
    p, a, nr, nz, plan, _, g = cone
    x = _vol(g, nz, 2, seed=5)
    got = _np(plan.fdk_adjoint(_t(x, cuda)))
    ref = orc.fdk_cone_adjoint(g, nr, nz, a, x)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)
    rng = np.random.default_rng(1)
    xx = rng.standard_normal((2, nz, g.ny, g.nx)).astype(np.float32)
    yy = rng.standard_normal((2, g.n_views, nr, g.n_cols)).astype(np.float32)
    ax = _np(plan.fdk_adjoint(_t(xx, cuda)))
    aty = _np(plan.fdk(_t(yy, cuda)))
    m = abs(float(np.vdot(ax, yy)) - float(np.vdot(xx, aty))) / (
        np.linalg.norm(ax) * np.linalg.norm(yy))
    assert m <= DOT_TOL, m


TRANSPOSE_CASES = {
    # 45 slices (six 8-slice lane groups, the last one ragged, in the
    # lanes-along-z kernel) on a detector a third as tall as the magnified
    # volume: samples clamp onto both edge rows
    "tall_clamped": lambda: G.cone_small(n=30, views=40, cols=60, n_rows=20, nz=45, pixel=6.0,
                                         dz=2.0, drow=3.0),
    # more detector rows than one view's accumulators fit in shared memory:
    # the row-block kernel
    "rows_beyond_shared_memory": lambda: G.cone_small(n=24, views=20, cols=64, n_rows=1000, nz=6,
                                                      drow=0.1),
}


@pytest.mark.parametrize("tex", [False, True])
@pytest.mark.parametrize("case", list(TRANSPOSE_CASES))
def test_fdk_adjoint_kernel_paths(cuda, orc, case, tex):
    """Both CB_EA transpose kernels against the oracle (texture weights: the
    filtered adjoint's 2e-3, as the fan-beam FBP adjoint) and the dot test."""
    p, a, nr, nz = TRANSPOSE_CASES[case]()
    plan = ConePlan(p, a, nr, nz, device=cuda, texture_weights=tex)
    g = orc.decode(p)
    x = _vol(g, nz, 2, seed=9)
    orc.set_texture_emulation(tex)
    try:
        ref = orc.fdk_cone_adjoint(g, nr, nz, a, x)
    finally:
        orc.set_texture_emulation(False)
    got = _np(plan.fdk_adjoint(_t(x, cuda)))
    assert rel_l2(got, ref) <= (2e-3 if tex else TOL), rel_l2(got, ref)
    rng = np.random.default_rng(2)
    xx = rng.standard_normal((2, nz, g.ny, g.nx)).astype(np.float32)
    yy = rng.standard_normal((2, g.n_views, nr, g.n_cols)).astype(np.float32)
    ax = _np(plan.fdk_adjoint(_t(xx, cuda)))
    aty = _np(plan.fdk(_t(yy, cuda)))
    m = abs(float(np.vdot(ax, yy)) - float(np.vdot(xx, aty))) / (
        np.linalg.norm(ax) * np.linalg.norm(yy))
    assert m <= DOT_TOL, m


def test_fdk_cone_single_row_matches_fan_fdk_op(cuda):
    p, a = G.fdk_driver(nview=60, nimg=48)
    cone = ConePlan(p, a, 1, 1, device=cuda)
    fan = FanPlan(p, a, device=cuda)
    y = torch.rand((2, 60, 888), device=cuda)
    v3 = cone.fdk(y.reshape(2, 60, 1, 888))
    v2 = fan.fdk_bp(y)
    assert rel_l2(_np(v3[:, 0]), _np(v2)) < 1e-6


def test_fdk_cone_autograd(cuda):
    from fanbeamctrecon_tensorflowop_gb300.autograd import fdk_cone
    p, a, nr, nz = G.cone_small(n=24, views=20, cols=48, n_rows=6, nz=5)
    plan = ConePlan(p, a, nr, nz, device=cuda)
    y = torch.rand((1, *plan.proj_shape), device=cuda, requires_grad=True)
    target = torch.rand((1, *plan.volume_shape), device=cuda)
    loss = 0.5 * ((fdk_cone(y, plan) - target) ** 2).sum()
    loss.backward()
    with torch.no_grad():
        expect = plan.fdk_adjoint(plan.fdk(y) - target)
    assert rel_l2(_np(y.grad), _np(expect)) < 1e-6


def test_cone_errors(cuda):
    p, a, nr, nz = G.cone_small()
    with pytest.raises(_lib.CtError):
        ConePlan(p, a, 0, nz, device=cuda)
    bad = p.copy()
    bad[14] = 0.0  # drow
    with pytest.raises(_lib.CtError):
        ConePlan(bad, a, nr, nz, device=cuda)
    plan = ConePlan(p, a, nr, nz, device=cuda)
    with pytest.raises(ValueError):
        plan.fdk(torch.zeros((1, 3, nr, 64), device=cuda))


def test_fdk_adjoint_high_dynamic_range(cuda, orc):
    """A volume that is one bright voxel on a faint background (four decades
    apart) through the FDK adjoint stays within tolerance, and zero gives zero."""
    p, a, nr, nz = G.cone_small(n=27, views=31, cols=57, n_rows=7, nz=9, pixel=6.6)
    plan = ConePlan(p, a, nr, nz, device=cuda)
    g = orc.decode(p)
    x = np.random.default_rng(8).uniform(0, 1e-3, (1, nz, g.ny, g.nx)).astype(np.float32)
    x[0, nz // 2, g.ny // 2, g.nx // 3] = 10.0
    got = _np(plan.fdk_adjoint(_t(x, cuda)))
    ref = orc.fdk_cone_adjoint(g, nr, nz, a, x)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)
    zero = plan.fdk_adjoint(torch.zeros((1, nz, g.ny, g.nx), device=cuda))
    assert float(zero.abs().max()) == 0.0


def test_cone_full_size_properties(cuda):
    """At the clinical cone size (512^2 x 64 voxels, 984 views of 888 x 64),
    properties that need no oracle: linearity of FDK and of the cone FP, the
    FDK adjoint's dot test, and that a volume in a batch equals the volume
    alone (tap images, fixed-point scale and quad images are per volume)."""
    p, a, nr, nz = G.config4()
    plan = ConePlan(p, a, nr, nz, device=cuda)
    gen = torch.Generator(device=cuda).manual_seed(0)
    y1 = torch.rand((2, *plan.proj_shape), device=cuda, generator=gen)
    y2 = torch.rand((2, *plan.proj_shape), device=cuda, generator=gen)
    f1, f2 = plan.fdk(y1), plan.fdk(y2)
    assert rel_l2(_np(plan.fdk(2.0 * y1 - 3.0 * y2)), _np(2.0 * f1 - 3.0 * f2)) < 1e-5
    assert torch.equal(plan.fdk(y1[1:2])[0], f1[1])
    x = torch.randn((2, *plan.volume_shape), device=cuda, generator=gen)
    yy = torch.randn((2, *plan.proj_shape), device=cuda, generator=gen)
    ax = plan.fdk_adjoint(x)
    aty = plan.fdk(yy)
    m = abs(float(torch.vdot(ax.double().flatten(), yy.double().flatten())) -
            float(torch.vdot(x.double().flatten(), aty.double().flatten()))) / (
        float(ax.double().norm()) * float(yy.double().norm()))
    assert m <= DOT_TOL, m
    assert torch.equal(plan.fdk_adjoint(x[1:2])[0], ax[1])
    v1 = torch.rand((2, *plan.volume_shape), device=cuda, generator=gen)
    p1 = plan.fp_cone(v1)
    p2 = plan.fp_cone(v1[1:2])
    assert torch.equal(p2[0], p1[1])
    assert rel_l2(_np(plan.fp_cone(3.0 * v1)), 3.0 * _np(p1)) < 1e-6


@pytest.mark.parametrize("n_rows", [40, 80, 128, 136])
def test_cone_fp_detector_heights(cuda, orc, n_rows):
    """The cone FP at 1 .. 4 detector rows per lane of the single-walk
    projector (40, 80, 128 rows) and past it (136 rows: the row-group
    projector), on the same 72 mm detector, against the oracle; rows cross
    several slices per segment at this cone angle."""
    p, a, nr, nz = G.cone_small(n=32, views=24, cols=48, n_rows=n_rows, nz=12,
                                drow=72.0 / n_rows)
    plan = ConePlan(p, a, nr, nz, device=cuda)
    g = orc.decode(p)
    x = _vol(g, nz, 1, seed=7)
    got = _np(plan.fp_cone(_t(x, cuda)))
    ref = orc.cone_fp(g, nr, nz, a, x)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)
    assert torch.equal(plan.fp_cone(_t(x, cuda)), plan.fp_cone(_t(x, cuda)))
