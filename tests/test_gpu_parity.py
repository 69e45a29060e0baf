"""Parity of the CUDA operators with the FP64 oracle, through the C ABI.

Tolerance (the contract): relative L2 error <= 1e-4 against the FP64 oracle
for every output; adjoint dot-product mismatch
|<Ax, y> - <x, A^T y>| / (||Ax|| ||y||) <= 1e-5."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import _lib, phantom
from fanbeamctrecon_tensorflowop_gb300.ops import FanPlan
import geometries as G

pytestmark = pytest.mark.gpu

TOL = 1e-4       # relative L2 vs the FP64 oracle
DOT_TOL = 1e-5   # adjoint dot-product mismatch

GEOMS = {
    "small": lambda: G.small(),
    "small_nonsquare_shift": lambda: G.small(n=50, ny=38, shift=1.5, views=72, cols=100),
    "odd_sizes": lambda: G.small(n=45, views=37, cols=61, pixel=3.9),
    "config0": G.config0,
}


def _images(g, batch, seed=0):
    out = []
    for b in range(batch):
        rfov = float(g.rfov)
        ell = phantom.random_ellipses(rfov, seed + b)
        out.append(phantom.rasterize(ell, g.nx, g.ny, float(g.dx), float(g.dy)))
    return np.stack(out)


def _sinos(g, batch, seed=0):
    return np.random.default_rng(seed).uniform(0, 1, (batch, g.n_views, g.n_cols)).astype(
        np.float32)


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)


def _np(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy().astype(np.float64)


@pytest.fixture(scope="module", params=list(GEOMS))
def case(request, cuda, orc):
    p, a = GEOMS[request.param]()
    plan = FanPlan(p, a, device=cuda)
    plan_sl = FanPlan(p, a, device=cuda, window=_lib.WINDOW_SHEPP_LOGAN)
    return request.param, p, a, plan, plan_sl, orc.decode(p)


def test_fp(case, cuda, orc):
    name, p, a, plan, _, g = case
    x = _images(g, 2)
    got = _np(plan.fp(_t(x, cuda)))
    ref = orc.fp_fan(g, a, x)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)


@pytest.mark.parametrize("batch", [9, 20])
def test_fp_staged_batches(case, cuda, orc, batch):
    """Batches of 8+ slices walk 16 (then 8, 4, 1) slices at a time: slices
    against the oracle (three of them) and against the slice projected alone."""
    name, p, a, plan, _, g = case
    x = _images(g, batch, seed=11)
    got = _np(plan.fp(_t(x, cuda)))
    pick = [0, batch // 2, batch - 1]
    ref = orc.fp_fan(g, a, x[pick])
    assert rel_l2(got[pick], ref) <= TOL, (name, rel_l2(got[pick], ref))
    for k in pick:
        alone = _np(plan.fp(_t(x[k:k + 1], cuda)))[0]
        assert np.array_equal(got[k], alone), (name, k)


def test_fp_adjoint(case, cuda, orc):
    name, p, a, plan, _, g = case
    y = _sinos(g, 2, seed=5)
    got = _np(plan.fp_adjoint(_t(y, cuda)))
    ref = orc.fp_fan_adjoint(g, a, y)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)


def test_bp_and_adjoint(case, cuda, orc):
    name, p, a, plan, _, g = case
    y = _sinos(g, 2, seed=1)
    got = _np(plan.bp(_t(y, cuda)))
    ref = orc.bp_fan(g, a, y)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)
    # 2 slices run one per thread, 6 four per thread with a ragged group of 2
    for nb in (2, 6):
        x = _images(g, nb, seed=7)
        got_t = _np(plan.bp_adjoint(_t(x, cuda)))
        ref_t = orc.bp_fan_transpose(g, a, x)
        assert rel_l2(got_t, ref_t) <= TOL, (nb, rel_l2(got_t, ref_t))
        # the same slice alone: the gather sums each slice in the same order
        assert np.array_equal(got_t[1], _np(plan.bp_adjoint(_t(x[1:2], cuda)))[0])


@pytest.mark.parametrize("nb", [4, 8, 13, 21])
def test_bp_fbp_tap_image_groups(case, cuda, orc, nb):
    """Batches of four or more read tap images: groups of eight slices per
    thread, then groups of four for the rest (the last one ragged).  Every
    slice equals the slice alone (one slice per thread, gathers) bit for bit,
    and the BP meets the oracle."""
    name, p, a, plan, plan_sl, g = case
    y = _sinos(g, nb, seed=3)
    yt = _t(y, cuda)
    for op in (plan.bp, plan.fbp, plan_sl.fbp):
        got = _np(op(yt))
        for b in sorted({0, nb // 2, nb - 1}):
            assert np.array_equal(got[b], _np(op(yt[b:b + 1]))[0]), (nb, b)
    ref = orc.bp_fan(g, a, y)
    got = _np(plan.bp(yt))
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)


@pytest.mark.parametrize("nb", [16, 40])
def test_transpose_slice_groups(case, cuda, orc, nb):
    """Batches of 16 and 40 slices through the BP / FBP transposes (four
    slices per thread, 40: ten groups).  Three slices against the oracle,
    each also against the one-slice path."""
    name, p, a, plan, _, g = case
    x = _images(g, nb, seed=9)
    pick = [0, nb // 2, nb - 1]
    for fn, oref in ((plan.bp_adjoint, orc.bp_fan_transpose),
                     (plan.fbp_adjoint, orc.fbp_fan_adjoint)):
        got = _np(fn(_t(x, cuda)))
        ref = oref(g, a, x[pick])
        assert rel_l2(got[pick], ref) <= TOL, (nb, rel_l2(got[pick], ref))
        for k in pick:
            alone = _np(fn(_t(x[k:k + 1], cuda)))[0]
            assert np.array_equal(got[k], alone), (k, rel_l2(got[k], alone))


def test_transpose_slice_groups_dot(case, cuda):
    name, p, a, plan, _, g = case
    rng = np.random.default_rng(12)
    x = rng.standard_normal((16, g.ny, g.nx)).astype(np.float32)
    y = rng.standard_normal((16, g.n_views, g.n_cols)).astype(np.float32)
    xt, yt = _t(x, cuda), _t(y, cuda)
    for k, (ax, aty) in {"bp": (plan.bp_adjoint(xt), plan.bp(yt)),
                         "fbp": (plan.fbp_adjoint(xt), plan.fbp(yt))}.items():
        m = _dot_mismatch(_np(ax), y.astype(np.float64), x.astype(np.float64), _np(aty))
        assert m <= DOT_TOL, (k, m)


@pytest.mark.parametrize("window", ["ramlak", "shepp_logan"])
def test_ramp_filter(case, cuda, orc, window):
    name, p, a, plan, plan_sl, g = case
    pl, w = (plan, orc.RAMLAK) if window == "ramlak" else (plan_sl, orc.SHEPP_LOGAN)
    y = _sinos(g, 2, seed=2)
    got = _np(pl.ramp_filter(_t(y, cuda)))
    ref = orc.ramp_filter(g, y, w)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)


@pytest.mark.parametrize("window", ["ramlak", "shepp_logan"])
def test_fbp_and_adjoint(case, cuda, orc, window):
    name, p, a, plan, plan_sl, g = case
    pl, w = (plan, orc.RAMLAK) if window == "ramlak" else (plan_sl, orc.SHEPP_LOGAN)
    x = _images(g, 2, seed=3)
    sino = orc.fp_fan(g, a, x)
    got = _np(pl.fbp(_t(sino, cuda)))
    ref = orc.fbp_fan(g, a, sino, w)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)
    got_t = _np(pl.fbp_adjoint(_t(x, cuda)))
    ref_t = orc.fbp_fan_adjoint(g, a, x, w)
    assert rel_l2(got_t, ref_t) <= TOL, rel_l2(got_t, ref_t)


def _dot_mismatch(ax, y, x, aty):
    lhs = float(np.vdot(ax, y))
    rhs = float(np.vdot(x, aty))
    return abs(lhs - rhs) / (np.linalg.norm(ax) * np.linalg.norm(y))


def test_adjoint_dot_products(case, cuda):
    name, p, a, plan, _, g = case
    rng = np.random.default_rng(11)
    x = rng.standard_normal((2, g.ny, g.nx)).astype(np.float32)
    y = rng.standard_normal((2, g.n_views, g.n_cols)).astype(np.float32)
    xt, yt = _t(x, cuda), _t(y, cuda)
    checks = {
        "fp": (plan.fp(xt), plan.fp_adjoint(yt)),
        "bp": (plan.bp_adjoint(xt), plan.bp(yt)),
        "fbp": (plan.fbp_adjoint(xt), plan.fbp(yt)),
    }
    for k, (ax, aty) in checks.items():
        m = _dot_mismatch(_np(ax), y.astype(np.float64), x.astype(np.float64), _np(aty))
        assert m <= DOT_TOL, (k, m)


def test_fdk_op(cuda, orc):
    """The reference FDK op's geometry (shift 1.125, rFOV 250), reduced views."""
    p, a = G.fdk_driver(nview=120, nimg=96)
    g = orc.decode(p)
    plan = FanPlan(p, a, device=cuda)
    y = _sinos(g, 2, seed=4)
    got = _np(plan.fdk_bp(_t(y, cuda)))
    ref = orc.fdk_bp(g, a, y)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)


def test_plain_loop_equals_fused(cuda):
    p, a = G.small(views=40)
    plan = FanPlan(p, a, device=cuda)
    g = plan.geom
    x = _t(_images(g, 2), cuda)
    y = _t(_sinos(g, 2), cuda)
    assert rel_l2(_np(plan.plain_fp(x)), _np(plan.fp(x))) < 1e-6
    assert rel_l2(_np(plan.plain_fp_adjoint(y)), _np(plan.fp_adjoint(y))) < 1e-6
    assert rel_l2(_np(plan.plain_bp(y)), _np(plan.bp(y))) < 1e-6


def test_finite_differences_and_oracle_gradient(cuda, orc):
    """Loss 0.5||FP(x) - y||^2: autograd gradient (hand-written adjoint) vs
    central differences (h = 1e-3) on 64 random pixels and vs the FP64 oracle
    gradient FP^T (FP x - y)."""
    from fanbeamctrecon_tensorflowop_gb300.autograd import forward_project
    p, a = G.small(n=48, views=60, cols=80)
    plan = FanPlan(p, a, device=cuda)
    g = orc.decode(p)
    x0 = _images(g, 1)[0]
    y = orc.fp_fan(g, a, _images(g, 1, seed=9))[0]
    x = _t(x0, cuda).requires_grad_(True)
    yt = torch.from_numpy(y).to(cuda)
    loss = 0.5 * ((forward_project(x, plan).double() - yt) ** 2).sum()
    loss.backward()
    grad = _np(x.grad)
    ref_grad = orc.fp_fan_adjoint(g, a, orc.fp_fan(g, a, x0) - y)[0]
    assert rel_l2(grad, ref_grad) <= TOL
    rng = np.random.default_rng(0)
    idx = rng.choice(g.nx * g.ny, 64, replace=False)
    h = 1e-3
    xf = _t(x0, cuda).reshape(-1)
    with torch.no_grad():
        for k in idx:
            xp = xf.clone(); xp[k] += h
            xm = xf.clone(); xm[k] -= h
            lp = 0.5 * ((plan.fp(xp.reshape(g.ny, g.nx))[0].double() - yt) ** 2).sum().item()
            lm = 0.5 * ((plan.fp(xm.reshape(g.ny, g.nx))[0].double() - yt) ** 2).sum().item()
            fd = (lp - lm) / (2 * h)
            gk = grad.reshape(-1)[k]
            assert abs(fd - gk) <= 1e-2 * max(1.0, abs(gk)), (k, fd, gk)


def test_errors_and_edge_cases(cuda):
    p, a = G.small()
    plan = FanPlan(p, a, device=cuda)
    lib = _lib.load()
    h = plan._h
    x = torch.zeros((1, *plan.image_shape), device=cuda)
    y = torch.zeros((1, *plan.sino_shape), device=cuda)
    s = torch.cuda.current_stream().cuda_stream
    # batch 0 is a no-op
    assert lib.ct_fp_fan(h, None, None, 0, None, 0, s) == 0
    # NULL buffers with work to do
    assert lib.ct_fp_fan(h, None, y.data_ptr(), 1, None, 0, s) == 2
    assert lib.ct_bp_fan(h, y.data_ptr(), None, 1, s) == 2
    # negative batch, aliasing
    assert lib.ct_fp_fan(h, x.data_ptr(), y.data_ptr(), -1, None, 0, s) == 1
    assert lib.ct_ramp_filter(h, y.data_ptr(), y.data_ptr(), 1, s) == 1
    # a workspace smaller than required
    need = plan.workspace_bytes(_lib.OP_FBP, 1)
    assert need == 4 * plan.geom.n_views * plan.geom.n_cols
    w = torch.empty(need, dtype=torch.uint8, device=cuda)
    assert lib.ct_fbp_fan(h, y.data_ptr(), x.data_ptr(), 1, w.data_ptr(), need - 4, s) == 3
    assert lib.ct_fbp_fan(h, y.data_ptr(), x.data_ptr(), 1, w.data_ptr(), need, s) == 0
    # shape / dtype / device checks of the torch layer
    with pytest.raises(ValueError):
        plan.fp(torch.zeros((1, 3, 3), device=cuda))
    with pytest.raises(TypeError):
        plan.fp(torch.zeros((1, *plan.image_shape), device=cuda, dtype=torch.float64))
    with pytest.raises(ValueError):
        plan.fp(torch.zeros((1, *plan.image_shape)))
    torch.cuda.synchronize()


def test_outputs_are_overwritten_not_accumulated(cuda):
    """Unlike the reference FDK op (unzeroed output, FDK/GPURecon_GPU.cu:237-238)."""
    p, a = G.small()
    plan = FanPlan(p, a, device=cuda)
    g = plan.geom
    y = _t(_sinos(g, 1), cuda)
    for fn in (plan.bp, plan.fbp, plan.fdk_bp, plan.fp_adjoint):
        out = torch.full((1, *plan.image_shape), 7.0, device=cuda)
        ref = fn(y)
        fn(y, out=out)
        assert torch.equal(out, ref) or rel_l2(_np(out), _np(ref)) < 1e-6


def test_deterministic_fp_and_bp(cuda):
    p, a = G.config0()
    plan = FanPlan(p, a, device=cuda)
    g = plan.geom
    x = _t(_images(g, 2), cuda)
    y = _t(_sinos(g, 2), cuda)
    assert torch.equal(plan.fp(x), plan.fp(x))
    assert torch.equal(plan.bp(y), plan.bp(y))
    assert torch.equal(plan.fbp(y), plan.fbp(y))
    # the transposes are gathers with a fixed summation order: no atomics
    assert torch.equal(plan.fp_adjoint(y), plan.fp_adjoint(y))
    assert torch.equal(plan.bp_adjoint(x), plan.bp_adjoint(x))
    assert torch.equal(plan.fbp_adjoint(x), plan.fbp_adjoint(x))


def test_utils_shim_numpy_and_torch(cuda):
    """The reference-named entry points: numpy in -> numpy out, CUDA tensors
    stay on device and carry gradients."""
    from fanbeamctrecon_tensorflowop_gb300 import utils
    p, a = G.small()
    plan = FanPlan(p, a, device=cuda)
    g = plan.geom
    img = _images(g, 3)
    vs, ps = [3, g.nx, g.ny], [3, g.n_views, g.n_cols]
    sino = utils.FP_module.fp_fan_curve(volume=img, angle=a, parameter=p, vol_shape=vs,
                                        proj_shape=ps)
    assert isinstance(sino, np.ndarray) and sino.shape == tuple(ps)
    np.testing.assert_array_equal(sino, plan.fp(_t(img, cuda)).cpu().numpy())
    rec = utils.load_op_library("./FBP/FBP.so").fbp_fan_curve(
        projection=sino, angle=a, parameter=p, vol_shape=vs, proj_shape=ps)
    assert rec.shape == tuple(vs)
    bp = utils.BP_module.bp_fan_curve(projection=torch.from_numpy(sino), angle=a, parameter=p,
                                      vol_shape=vs, proj_shape=ps)
    assert isinstance(bp, torch.Tensor) and not bp.is_cuda
    fdk = utils.load_op_library("./FBP_op.so").BackProjection(
        projection=sino[:1], angle=a, parameter=p, vol_shape=[1, g.nx, g.ny],
        proj_shape=[1, g.n_views, g.n_cols])
    np.testing.assert_allclose(fdk, rec[:1], rtol=0, atol=1e-6 * np.abs(rec).max())
    xt = _t(img, cuda).requires_grad_(True)
    out = utils.fp_fan_curve(volume=xt, angle=a, parameter=p, vol_shape=vs, proj_shape=ps)
    assert out.is_cuda and out.requires_grad
    out.sum().backward()
    assert xt.grad is not None and torch.isfinite(xt.grad).all()


def test_utils_large_host_batches(cuda):
    """The reference-named entry points on a 40-slice host batch (numpy and
    CPU tensors) equal the device-resident operators bit for bit; a shape
    attribute that does not hold the result is refused."""
    from fanbeamctrecon_tensorflowop_gb300 import utils
    p, a = G.small()
    plan = FanPlan(p, a, device=cuda)
    g = plan.geom
    nb = 40
    img = _images(g, nb, seed=3)
    sino = _sinos(g, nb, seed=4)
    vs, ps = [nb, g.nx, g.ny], [nb, g.n_views, g.n_cols]
    kw = dict(angle=a, parameter=p, vol_shape=vs, proj_shape=ps)
    got = utils.fp_fan_curve(volume=img, **kw)
    assert isinstance(got, np.ndarray) and got.shape == tuple(ps)
    np.testing.assert_array_equal(got, plan.fp(_t(img, cuda)).cpu().numpy())
    got = utils.bp_fan_curve(projection=torch.from_numpy(sino), **kw)
    assert isinstance(got, torch.Tensor) and not got.is_cuda and got.shape == tuple(vs)
    np.testing.assert_array_equal(got.numpy(), plan.bp(_t(sino, cuda)).cpu().numpy())
    got = utils.fbp_fan_curve(projection=sino, **kw)
    np.testing.assert_array_equal(got, plan.fbp(_t(sino, cuda)).cpu().numpy())
    got = utils.back_projection(projection=sino, **kw)
    np.testing.assert_array_equal(got, plan.fdk_bp(_t(sino, cuda)).cpu().numpy())
    with pytest.raises(ValueError):
        utils.fp_fan_curve(volume=img, angle=a, parameter=p, vol_shape=vs,
                           proj_shape=[nb - 1, g.n_views, g.n_cols])


def test_config1_against_oracle(cuda, orc):
    """The clinical-scale geometry (512^2, 984 x 888): FP of the seeded
    phantom, Shepp-Logan FBP of that sinogram, BP of a U[0,1) sinogram."""
    p, a = G.config1()
    g = orc.decode(p)
    plan = FanPlan(p, a, device=cuda, window=_lib.WINDOW_SHEPP_LOGAN)
    x = phantom.ellipse_phantom(512, 0.7, seed=0)[None]
    sino = _np(plan.fp(_t(x, cuda)))
    ref = orc.fp_fan(g, a, x)
    assert rel_l2(sino, ref) <= TOL, rel_l2(sino, ref)
    rec = _np(plan.fbp(_t(ref, cuda)))
    ref_rec = orc.fbp_fan(g, a, ref, orc.SHEPP_LOGAN)
    assert rel_l2(rec, ref_rec) <= TOL, rel_l2(rec, ref_rec)
    y = _sinos(g, 1, seed=3)
    got = _np(plan.bp(_t(y, cuda)))
    assert rel_l2(got, orc.bp_fan(g, a, y)) <= TOL


def test_full_size_batch_properties(cuda):
    """At the batch-32 clinical size, properties that need no oracle:
    linearity of FP and FBP, the FP dot test, and slice independence."""
    p, a = G.config1()
    plan = FanPlan(p, a, device=cuda)
    g = plan.geom
    B = 32
    gen = torch.Generator(device=cuda).manual_seed(0)
    x1 = torch.rand((B, g.ny, g.nx), device=cuda, generator=gen)
    x2 = torch.rand((B, g.ny, g.nx), device=cuda, generator=gen)
    y = torch.randn((B, g.n_views, g.n_cols), device=cuda, generator=gen)
    f1, f2 = plan.fp(x1), plan.fp(x2)
    f12 = plan.fp(2.0 * x1 - 3.0 * x2)
    assert rel_l2(_np(f12), _np(2.0 * f1 - 3.0 * f2)) < 1e-5
    m = _dot_mismatch(_np(f1), _np(y), _np(x1), _np(plan.fp_adjoint(y)))
    assert m <= DOT_TOL, m
    # slice b of a batch equals the slice alone (same arithmetic per slice
    # whatever the number of slices per walk)
    assert torch.equal(plan.fp(x1[5:6])[0], f1[5])
    r = plan.fbp(y)
    assert torch.equal(plan.fbp(y[7:8])[0], r[7])
