"""Plans with texture_weights = 1: the backprojectors interpolate with the GPU
texture unit's 8-bit weights, as the reference's texture fetches did.

Checked against the executed reference's golden vectors (refgold), against
the FP64 oracle in texture-emulation mode, and for exact adjointness.  What
separates the kernels from the reference then is only FP32 rounding of the
column and row coordinates moving a weight across a 1/256 boundary.  The
ramp filter amplifies such a step on noise-like data (FBP of U[0,1)
sinograms sits ~3e-4 from the emulating oracle), so the filtered operators
are compared on projections of phantoms, as the reference is used.  The
filtered adjoints filter the transposed backprojection, so they amplify the
same steps whatever the input: FBP and FDK adjoints are held to 2e-3 of the
emulating oracle (measured 6.9e-4 and 1.9e-4) and to exactness by the
dot-product test.
Tolerances (relative L2): against the executed reference BP 2e-5, BP of
U[0,1) noise 1e-4, FBP and FDK 1e-4; against the texture-emulating oracle
1e-4 (filtered adjoints 2e-3); adjoint dot-product mismatch 1e-5."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import _lib, phantom
from fanbeamctrecon_tensorflowop_gb300.batch import UnevenBatch
from fanbeamctrecon_tensorflowop_gb300.ops import ConePlan, FanPlan
from refgold import CASES, gold, reference_view
import geometries as G

pytestmark = pytest.mark.gpu

REF_TOL = {"bp": 2e-5, "bp_noise": 1e-4, "fbp": 1e-4, "fdk": 1e-4}
TOL = 1e-4
ADJ_TOL = {"fbp_adjoint": 2e-3, "fdk_adjoint": 2e-3}
DOT_TOL = 1e-5


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)


def _np(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy().astype(np.float64)


@pytest.fixture
def texture_oracle(orc):
    orc.set_texture_emulation(True)
    try:
        yield orc
    finally:
        orc.set_texture_emulation(False)


@pytest.mark.parametrize("case", CASES)
def test_texture_mode_matches_executed_reference(cuda, case):
    p, a = gold(case, "parameter"), gold(case, "angle")
    plan = FanPlan(p, a, device=cuda, texture_weights=True)
    exact = FanPlan(p, a, device=cuda)
    fp_in = _t(gold(case, "fp"), cuda)
    got = {"bp": plan.bp(fp_in), "fbp": plan.fbp(fp_in), "fdk": plan.fdk_bp(fp_in),
           "bp_noise": plan.bp(_t(gold(case, "noise"), cuda))}
    errs = {op: rel_l2(reference_view(case, op, _np(y)), gold(case, op)) for op, y in got.items()}
    print(case, {k: f"{v:.2e}" for k, v in errs.items()})
    for op, e in errs.items():
        assert e <= REF_TOL[op], f"{case}/{op}: {e:.3e}"
    # the mode changes the result (the exact weights sit 1e-4 away in FBP)
    assert rel_l2(_np(exact.fbp(fp_in)), _np(got["fbp"])) > 1e-6


def test_texture_mode_against_oracle_and_adjoints(cuda, texture_oracle):
    orc = texture_oracle
    p, a = G.small(n=50, ny=38, shift=1.5, views=72, cols=100)
    g = orc.decode(p)
    plan = FanPlan(p, a, device=cuda, texture_weights=True)
    rng = np.random.default_rng(3)
    y = rng.uniform(0, 1, (2, g.n_views, g.n_cols)).astype(np.float32)
    x = np.stack([phantom.ellipse_phantom(g.nx, float(g.dx), seed=s, ny=g.ny) for s in (0, 1)])
    ys = orc.fp_fan(g, a, x).astype(np.float32)  # projections of phantoms
    for name, got, ref in (
            ("bp", plan.bp(_t(y, cuda)), orc.bp_fan(g, a, y)),
            ("fbp", plan.fbp(_t(ys, cuda)), orc.fbp_fan(g, a, ys)),
            ("fdk", plan.fdk_bp(_t(ys, cuda)), orc.fdk_bp(g, a, ys)),
            ("bp_adjoint", plan.bp_adjoint(_t(x, cuda)), orc.bp_fan_transpose(g, a, x)),
            ("fbp_adjoint", plan.fbp_adjoint(_t(x, cuda)), orc.fbp_fan_adjoint(g, a, x))):
        e = rel_l2(_np(got), ref)
        print(name, f"{e:.2e}")
        assert e <= ADJ_TOL.get(name, TOL), (name, e)
    xx = rng.standard_normal((2, g.ny, g.nx)).astype(np.float32)
    yy = rng.standard_normal((2, g.n_views, g.n_cols)).astype(np.float32)
    for fwd, adj in ((plan.bp, plan.bp_adjoint), (plan.fbp, plan.fbp_adjoint)):
        ax = _np(adj(_t(xx, cuda)))
        aty = _np(fwd(_t(yy, cuda)))
        m = abs(float(np.vdot(ax, yy)) - float(np.vdot(xx, aty))) / (
            np.linalg.norm(ax) * np.linalg.norm(yy))
        assert m <= DOT_TOL, m


def test_texture_mode_transpose_slice_groups(cuda, texture_oracle):
    """BP and its transpose on 16 slices with the texture weights (the BP in
    groups of eight slices from tap images): two slices of each against the
    emulating oracle, dot test."""
    orc = texture_oracle
    p, a = G.small(n=50, ny=38, shift=1.5, views=72, cols=100)
    g = orc.decode(p)
    plan = FanPlan(p, a, device=cuda, texture_weights=True)
    x = np.stack([phantom.ellipse_phantom(g.nx, float(g.dx), seed=s, ny=g.ny)
                  for s in range(16)]).astype(np.float32)
    got = _np(plan.bp_adjoint(_t(x, cuda)))
    e = rel_l2(got[[0, 15]], orc.bp_fan_transpose(g, a, x[[0, 15]]))
    assert e <= TOL, e
    y16 = np.random.default_rng(9).uniform(0, 1, (16, g.n_views, g.n_cols)).astype(np.float32)
    got = _np(plan.bp(_t(y16, cuda)))
    e = rel_l2(got[[0, 15]], orc.bp_fan(g, a, y16[[0, 15]]))
    assert e <= ADJ_TOL.get("bp", TOL), e
    rng = np.random.default_rng(5)
    xx = rng.standard_normal((16, g.ny, g.nx)).astype(np.float32)
    yy = rng.standard_normal((16, g.n_views, g.n_cols)).astype(np.float32)
    ax = _np(plan.bp_adjoint(_t(xx, cuda)))
    aty = _np(plan.bp(_t(yy, cuda)))
    m = abs(float(np.vdot(ax, yy)) - float(np.vdot(xx, aty))) / (
        np.linalg.norm(ax) * np.linalg.norm(yy))
    assert m <= DOT_TOL, m


def test_texture_mode_cone(cuda, texture_oracle):
    orc = texture_oracle
    p, a, nr, nz = G.cone_small()
    g = orc.decode(p)
    plan = ConePlan(p, a, nr, nz, device=cuda, texture_weights=True)
    rng = np.random.default_rng(4)
    y = rng.uniform(0, 1, (1, g.n_views, nr, g.n_cols)).astype(np.float32)
    sl = phantom.ellipse_phantom(g.nx, float(g.dx), seed=2, ny=g.ny)
    x = (sl[None] * (1.0 + 0.3 * np.sin(np.linspace(0, 3, nz)))[:, None, None])[None]
    x = x.astype(np.float32)
    ys = orc.cone_fp(g, nr, nz, a, x).astype(np.float32)  # projections of a phantom
    for name, got, ref in (
            ("cone_bp", plan.cone_bp(_t(y, cuda)), orc.cone_bp(g, nr, nz, a, y)),
            ("fdk", plan.fdk(_t(ys, cuda)), orc.fdk_cone(g, nr, nz, a, ys)),
            ("fdk_adjoint", plan.fdk_adjoint(_t(x, cuda)), orc.fdk_cone_adjoint(g, nr, nz, a, x))):
        e = rel_l2(_np(got), ref)
        print(name, f"{e:.2e}")
        assert e <= ADJ_TOL.get(name, TOL), (name, e)
    xx = rng.standard_normal(x.shape).astype(np.float32)
    yy = rng.standard_normal(y.shape).astype(np.float32)
    ax = _np(plan.fdk_adjoint(_t(xx, cuda)))
    aty = _np(plan.fdk(_t(yy, cuda)))
    m = abs(float(np.vdot(ax, yy)) - float(np.vdot(xx, aty))) / (
        np.linalg.norm(ax) * np.linalg.norm(yy))
    assert m <= DOT_TOL, m


def test_texture_mode_rejected_where_unsupported(cuda):
    p, a = G.small()
    plan = FanPlan(p, a, device=cuda, texture_weights=True)
    g = plan.geom
    sino = torch.zeros(g.n_views, g.n_cols, device=cuda)
    img = torch.zeros(g.ny, g.nx, device=cuda)
    with pytest.raises(_lib.CtError):
        UnevenBatch([(plan, "bp", sino, img)]).run()
    with pytest.raises(_lib.CtError):
        plan.plain_bp(sino[None])
    # the forward projector is exact in both modes, and batches accept it
    UnevenBatch([(plan, "fp", img, sino)]).run()
