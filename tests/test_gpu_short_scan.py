"""Short-scan (Parker-weighted) FBP / FDK and their adjoints on the GPU
against the FP64 oracle, through the C ABI.  Tolerances as for the full-scan
operators: relative L2 <= 1e-4, adjoint dot-product mismatch <= 1e-5."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2
from fanbeamctrecon_tensorflowop_gb300 import _lib, phantom
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


def _dot_mismatch(ax, y, x, aty):
    return abs(float(np.vdot(ax, y)) - float(np.vdot(x, aty))) / (
        np.linalg.norm(ax) * np.linalg.norm(y))


CASES = {
    # C % 4 == 0: the tensor-core filter; C % 4 == 2: the direct filter
    "tc_filter": dict(n=64, views=120, cols=192, pixel=4.0, dcol=4.0 * G.DCOL),
    "direct_filter": dict(n=45, views=97, cols=130, pixel=5.7, dcol=4.0 * G.DCOL, shift=1.25),
    "reversed": dict(n=64, views=120, cols=192, pixel=4.0, dcol=4.0 * G.DCOL, reverse=True),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("window", [_lib.WINDOW_RAMLAK, _lib.WINDOW_SHEPP_LOGAN])
def test_short_scan_fbp_fdk_and_adjoint(name, window, cuda, orc):
    p, a = G.short_scan(**CASES[name])
    plan = FanPlan(p, a, device=cuda, window=window, short_scan=True)
    g = orc.decode(p)
    rng = np.random.default_rng(7)
    y = rng.uniform(0, 1, (2, g.n_views, g.n_cols)).astype(np.float32)
    x = rng.standard_normal((2, g.ny, g.nx)).astype(np.float32)
    got = _np(plan.fbp(_t(y, cuda)))
    ref = orc.fbp_fan(g, a, y, window, short_scan=True)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)
    got = _np(plan.fdk_bp(_t(y, cuda)))
    ref = orc.fdk_bp(g, a, y, window, short_scan=True)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)
    ax = _np(plan.fbp_adjoint(_t(x, cuda)))
    ref = orc.fbp_fan_adjoint(g, a, x, window, short_scan=True)
    assert rel_l2(ax, ref) <= TOL, rel_l2(ax, ref)
    aty = _np(plan.fbp(_t(y, cuda)))
    assert _dot_mismatch(ax, y, x, aty) <= DOT_TOL


def test_short_scan_recovers_disc_and_differs_from_full_scan(cuda, orc):
    p, a = G.short_scan(views=200)
    g = orc.decode(p)
    mu, rad, cx, cy = 0.02, 0.35 * g.rfov, 0.2 * g.rfov, -0.1 * g.rfov
    ell = np.array([[cx, cy, rad, rad, 0.0, mu]])
    p0, u = phantom.fan_rays(g.sid, a, g.left, g.dcol, g.n_cols)
    sino = phantom.ellipse_line_integrals(ell, p0, u)
    x = g.xmin + g.dx * (np.arange(g.nx) + 0.5)
    r = np.sqrt((x[None, :] - cx) ** 2 + (x[:, None] - cy) ** 2)
    interior = r < 0.7 * rad
    rec = _np(FanPlan(p, a, device=cuda, short_scan=True).fbp(_t(sino, cuda)))[0]
    assert abs(rec[interior].mean() / mu - 1.0) < 0.005
    plain = _np(FanPlan(p, a, device=cuda).fbp(_t(sino, cuda)))[0]
    assert abs(plain[interior].mean() / mu - 1.0) > 0.3


def test_short_scan_cone_fdk_and_adjoint(cuda, orc):
    nr, nz, drow = 10, 8, 6.0
    p, a = G.short_scan(n=32, views=64, cols=64, pixel=5.6, dcol=4.0 * G.DCOL,
                        det_bottom=-nr * drow / 2.0, drow=drow, dz=3.0)
    plan = ConePlan(p, a, nr, nz, device=cuda, short_scan=True)
    g = orc.decode(p)
    rng = np.random.default_rng(2)
    y = rng.uniform(0, 1, (2, g.n_views, nr, g.n_cols)).astype(np.float32)
    x = rng.standard_normal((2, nz, g.ny, g.nx)).astype(np.float32)
    got = _np(plan.fdk(_t(y, cuda)))
    ref = orc.fdk_cone(g, nr, nz, a, y, short_scan=True)
    assert rel_l2(got, ref) <= TOL, rel_l2(got, ref)
    ax = _np(plan.fdk_adjoint(_t(x, cuda)))
    ref = orc.fdk_cone_adjoint(g, nr, nz, a, x, short_scan=True)
    assert rel_l2(ax, ref) <= TOL, rel_l2(ax, ref)
    assert _dot_mismatch(ax, y, x, _np(plan.fdk(_t(y, cuda)))) <= DOT_TOL


def test_short_scan_in_uneven_batch(cuda):
    items, ref = [], []
    for k, op in enumerate(("fbp", "fbp_adjoint", "fbp", "bp")):
        p, a = G.short_scan(n=48 + 16 * k, views=90 + 10 * k, cols=128 + 32 * k, pixel=4.0,
                            dcol=4.0 * G.DCOL)
        plan = FanPlan(p, a, device=cuda, short_scan=(k != 2))
        g = plan.geom
        x = (torch.rand(plan.image_shape, device=cuda) if op == "fbp_adjoint"
             else torch.rand(plan.sino_shape, device=cuda))
        y = torch.full(plan.sino_shape if op == "fbp_adjoint" else plan.image_shape,
                       float("nan"), device=cuda)
        items.append((plan, op, x, y))
        ref.append({"fbp": plan.fbp, "fbp_adjoint": plan.fbp_adjoint, "bp": plan.bp}[op](x)[0])
    UnevenBatch(items).run()
    for (plan, op, x, y), want in zip(items, ref):
        assert rel_l2(_np(y), _np(want)) <= 1e-5, op


def test_short_scan_option_validation(cuda):
    p, a = G.short_scan(n=32, views=40, cols=64)
    plan = FanPlan(p, a, device=cuda, short_scan=True)
    lib = _lib.load()
    stream = torch.cuda.current_stream(cuda).cuda_stream
    sino = torch.zeros(plan.sino_shape, device=cuda)
    img = torch.zeros(plan.image_shape, device=cuda)
    # the static-scratch entry point has room for one sinogram only
    assert lib.ct_fbp_fan_static_scratch(plan._h, sino.data_ptr(), img.data_ptr(), 1,
                                         stream) == 6  # CT_ERR_UNSUPPORTED
    assert b"short-scan" in lib.ct_last_error()
    import ctypes
    opts = _lib.CtPlanOpts()
    opts.short_scan = 2
    h = ctypes.c_void_p()
    st = lib.ct_plan_create(ctypes.byref(plan.geom),
                            plan.angles.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                            int(plan.angles.shape[0]), ctypes.byref(opts), ctypes.byref(h))
    assert st == 1 and not h.value
