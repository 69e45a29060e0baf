"""Oracle comparisons at the workloads' own clinical sizes (through the C ABI).

- The FP adjoint at 512^2 / 984 x 888 against the FP64 oracle's transpose of
  the ray march (FP/transform.cu:103-146 transposed), on a sinogram that is
  nonzero on every 4th view (the oracle's cost; the kernel runs every view).
- The batch-32 differentiable step: the gradient of 0.5||FP(x) - y||^2 for a
  slice of the batch against central differences on 64 random pixels and
  against the FP64 oracle gradient FP^T(FP x - y), at 512^2 / 984 x 888.
- Cone beam at 512^2 x 64 voxels with the 888 x 64 detector (8 views): the
  cone FP, FDK and FDK adjoint against the oracle (FDK/GPURecon_GPU.cu:15-50
  restated, with its ramp filter), on the seeded ellipsoid phantom.
Tolerances as everywhere: relative L2 <= 1e-4, dot mismatch <= 1e-5."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import phantom
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


@pytest.fixture(scope="module")
def c1(cuda, orc):
    p, a = G.config1()
    return p, a, FanPlan(p, a, device=cuda), orc.decode(p)


def test_fp_adjoint_clinical_against_oracle(cuda, orc, c1):
    p, a, plan, g = c1
    sel = np.arange(0, g.n_views, 4)
    sub = orc.OrcGeom.from_buffer_copy(g)
    sub.n_views = len(sel)
    y = np.random.default_rng(5).standard_normal((1, g.n_views, g.n_cols)).astype(np.float32)
    ym = np.zeros_like(y)
    ym[:, sel] = y[:, sel]
    got = _np(plan.fp_adjoint(_t(ym, cuda)))
    ref = orc.fp_fan_adjoint(sub, a[sel], y[:, sel])
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)


@pytest.mark.parametrize("window", ["ramlak", "shepp_logan"])
def test_bp_and_fbp_adjoint_clinical_against_oracle(cuda, orc, c1, window):
    """The BP transpose and the FBP adjoint at 512^2 / 984 x 888 on the seeded
    phantom.  The FBP adjoint ends with the ramp filter, which amplifies the
    transpose's per-pixel column errors about 80-fold: the gather form keeps
    them at ~1e-7 of a channel."""
    from fanbeamctrecon_tensorflowop_gb300 import _lib
    p, a, plan, g = c1
    win = _lib.WINDOW_SHEPP_LOGAN if window == "shepp_logan" else _lib.WINDOW_RAMLAK
    plan_w = FanPlan(p, a, device=cuda, window=win)
    x = phantom.phantom_batch(2, 512, 0.7, seed0=4)
    got = _np(plan_w.fbp_adjoint(_t(x, cuda)))
    ref = orc.fbp_fan_adjoint(g, a, x[:1], window=orc.SHEPP_LOGAN if window == "shepp_logan"
                              else orc.RAMLAK)
    assert rel_l2(got[:1], ref) <= TOL, rel_l2(got[:1], ref)
    if window == "ramlak":
        got = _np(plan.bp_adjoint(_t(x, cuda)))
        ref = orc.bp_fan_transpose(g, a, x[1:2])
        assert rel_l2(got[1:2], ref) <= TOL, rel_l2(got[1:2], ref)


def test_batch32_gradient_clinical(cuda, orc, c1):
    """Config 2: batch of 32 clinical slices, y = FP(phantom) + N(0, (0.01 max)^2)."""
    from fanbeamctrecon_tensorflowop_gb300.autograd import forward_project
    p, a, plan, g = c1
    B = 32
    x0 = phantom.phantom_batch(B, 512, 0.7, seed0=0)
    truth = phantom.phantom_batch(B, 512, 0.7, seed0=100)
    with torch.no_grad():
        yt = plan.fp(_t(truth, cuda)).double()
        yt += 0.01 * float(yt.abs().max()) * torch.randn(
            yt.shape, device=cuda, dtype=torch.float64,
            generator=torch.Generator(device=cuda).manual_seed(0))
    x = _t(x0, cuda).requires_grad_(True)
    loss = 0.5 * ((forward_project(x, plan).double() - yt) ** 2).sum()
    loss.backward()
    grad = _np(x.grad)
    # the oracle gradient of slice 3
    k = 3
    y3 = yt[k].cpu().numpy()
    ref = orc.fp_fan_adjoint(g, a, orc.fp_fan(g, a, x0[k:k + 1])[0] - y3)[0]
    assert rel_l2(grad[k], ref) <= TOL, rel_l2(grad[k], ref)
    # central differences of the batch loss on 64 random pixels of slice k
    rng = np.random.default_rng(1)
    inside = np.flatnonzero(np.abs(x0[k]).reshape(-1) > 0)
    idx = rng.choice(inside, 64, replace=False)
    h = 1e-2  # the loss is quadratic: central differences are exact up to rounding
    xf = _t(x0[k], cuda).reshape(-1)
    yk = yt[k]
    with torch.no_grad():
        for i in idx:
            xp = xf.clone()
            xp[i] += h
            xm = xf.clone()
            xm[i] -= h
            lp = 0.5 * ((plan.fp(xp.reshape(512, 512))[0].double() - yk) ** 2).sum().item()
            lm = 0.5 * ((plan.fp(xm.reshape(512, 512))[0].double() - yk) ** 2).sum().item()
            fd = (lp - lm) / (2 * h)
            gi = grad[k].reshape(-1)[i]
            assert abs(fd - gi) <= 1e-2 * max(1.0, abs(gi)), (i, fd, gi)


@pytest.fixture(scope="module")
def c4(cuda, orc):
    p, a, nr, nz = G.config4(views=8)
    return p, a, nr, nz, ConePlan(p, a, nr, nz, device=cuda), orc.decode(p)


def test_cone_clinical_against_oracle(cuda, orc, c4):
    p, a, nr, nz, plan, g = c4
    vol = phantom.ellipsoid_phantom(512, nz, 0.7, 0.625, seed=0)[None]
    proj = _np(plan.fp_cone(_t(vol, cuda)))
    ref = orc.cone_fp(g, nr, nz, a, vol)
    assert rel_l2(proj, ref) <= TOL, rel_l2(proj, ref)
    rec = _np(plan.fdk(_t(ref, cuda)))
    ref_rec = orc.fdk_cone(g, nr, nz, a, ref)
    assert rel_l2(rec, ref_rec) <= TOL, rel_l2(rec, ref_rec)
    adj = _np(plan.fdk_adjoint(_t(vol, cuda)))
    ref_adj = orc.fdk_cone_adjoint(g, nr, nz, a, vol)
    assert rel_l2(adj, ref_adj) <= TOL, rel_l2(adj, ref_adj)


def test_cone_clinical_dot(cuda, c4):
    p, a, nr, nz, plan, g = c4
    gen = torch.Generator(device=cuda).manual_seed(2)
    x = torch.randn((1, *plan.volume_shape), device=cuda, generator=gen)
    y = torch.randn((1, *plan.proj_shape), device=cuda, generator=gen)
    ax, aty = plan.fdk_adjoint(x).double(), plan.fdk(y).double()
    m = abs(float((ax * y.double()).sum()) - float((x.double() * aty).sum())) / (
        float(ax.norm()) * float(y.double().norm()))
    assert m <= DOT_TOL, m
